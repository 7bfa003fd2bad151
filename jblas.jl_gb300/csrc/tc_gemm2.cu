// Slice-product engine, CTA-pair form: tcgen05.mma.cta_group::2 on 256 x 256 output tiles.
//
// Two CTAs of a cluster (on the two SMs of a TPC) share one tile: CTA r holds rows
// [m0 + 128 r, m0 + 128 r + 128) of the A planes and rows [n0 + 128 r, ...) of the B
// planes, so each SM loads half of B.  Per 64-wide K panel an SM then takes 32 KB instead
// of the 48 KB of the single-CTA 128 x 256 tile, for the same tensor work per SM; the freed
// shared memory gives 6 pipeline stages instead of 4.
//
//   warp 0      TMA producer in both CTAs; copies land in the CTA's own shared memory and
//               are counted on the LEADER's (rank 0) full barrier
//   warp 1      TMEM allocation (both CTAs, pair-wide); in the leader one lane issues the
//               M = 256, N = 256 MMAs and commits to the barriers of both CTAs
//   warps 2-9   epilogue in both CTAs (warps 2-17 for the CRT epilogue): each CTA drains its
//               128 rows x 256 columns, as the single-CTA kernel (tc_gemm.cu) does, and every
//               epilogue warp arrives on the leader's tmem_empty
// Waits are bounded as in tc_gemm.cu; both CTAs meet at a cluster barrier before TMEM is
// released.
#include <cuda_bf16.h>

#include "gb_common.cuh"
#include "profile.cuh"
#include "tc_gemm.cuh"

namespace gb {

// Threads per CTA: 2 role warps + 8 epilogue warps, or 16 for the CRT epilogue, whose drains
// come every 16 K panels and need more warps to hide their latency (4 per TMEM lane quadrant,
// 64 columns each; 96 registers per thread fit 18 warps).
template <int EPI>
struct P2Shape {
  static constexpr int THREADS = (EPI == TC_EPI_CRT) ? 576 : 320;
  static constexpr int EPI_WARPS = THREADS / 32 - 2;
  static constexpr int COLS = TC_BN / (EPI_WARPS / 4);   // columns per epilogue warp
};
constexpr int P2_STAGES = 6;
constexpr int P2_A_BYTES = 128 * TC_BK * 2;     // 16 KB: this CTA's 128 rows of A
constexpr int P2_B_BYTES = 128 * TC_BK * 2;     // 16 KB: this CTA's half of B
constexpr int P2_STAGE_BYTES = P2_A_BYTES + P2_B_BYTES;
constexpr int P2_TMEM_COLS = 512;
constexpr int P2_SMEM_BYTES = P2_STAGES * P2_STAGE_BYTES + 1024 + 256;
// TC_EPI_F32 with TMA stores: behind the stages and a 1 KB barrier block, one 32 x 32 FP32 box
// of C per epilogue warp (8 warps x 4 KB), in the tensor map's own layout (rows fastest): a warp
// writes 32 consecutive floats per column, so the staging is conflict-free without a swizzle.
constexpr int P2_CSTAGE_OFF = P2_STAGES * P2_STAGE_BYTES + 1024;
constexpr int P2_CSTAGE_BYTES = 8 * 32 * 32 * 4;
constexpr int P2_SMEM_BYTES_F32 = 1024 + P2_CSTAGE_OFF + P2_CSTAGE_BYTES;
static_assert(P2_SMEM_BYTES_F32 <= 232448, "shared memory per CTA");

constexpr int P2_EXP_NONFINITE = 0x7FFFFFFF;
constexpr uint64_t P2_CLEANUP_WAIT_NS = 2000000000ull;

__device__ __forceinline__ void p2_tile_coords(int t, int tiles_m, int tiles_n, int GM, int& tm, int& tn) {
  // bands of GM pair tiles (GM x 256 rows; 8 by default), column tiles inside a band
  const int band = t / (GM * tiles_n);
  const int in_band = t - band * GM * tiles_n;
  const int band_rows = min(GM, tiles_m - band * GM);
  tm = band * GM + in_band % band_rows;
  tn = in_band / band_rows;
}

__device__ __forceinline__ double p2_exact_int_f32_times_pow2(uint32_t u, unsigned long long wbias) {
  const unsigned long long sign = static_cast<unsigned long long>(u & 0x80000000u) << 32;
  const uint32_t mag = u & 0x7FFFFFFFu;
  const unsigned long long body = mag ? ((static_cast<unsigned long long>(mag) + wbias) << 29) : 0ull;
  return __longlong_as_double(static_cast<long long>(sign | body));
}

// Work units: a whole tile (all groups) or, for TC_EPI_CRT, one (tile, modulus) pair,
// modulus-major, so the last round of a persistent grid is nearly full (1024 tiles x 15
// moduli over 76 clusters: 99.6% instead of 96%) and concurrently active units share the
// same modulus' planes.
template <int EPI>
__device__ __forceinline__ void p2_unit(int u, int ntiles, int G, int& t, int& g0, int& g1) {
  if (EPI == TC_EPI_CRT) {
    g0 = u / ntiles;
    g1 = g0 + 1;
    t = u - g0 * ntiles;
  } else {
    t = u;
    g0 = 0;
    g1 = G;
  }
}

// TcProblem fields are reused with pair tiles: tiles_m = ceil(M / 256), tiles_n = ceil(N / 256),
// tile_begin in pair-tile units.
__device__ __forceinline__ int p2_problem_of(const TcParams& prm, int t) {
  return (prm.nprob == 2 && t >= prm.prob[1].tile_begin) ? 1 : 0;
}

template <int EPI>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(P2Shape<EPI>::THREADS, 1)
    tc_gemm_pair_kernel(const __grid_constant__ CUtensorMap tmap_a0, const __grid_constant__ CUtensorMap tmap_b0,
                        const __grid_constant__ CUtensorMap tmap_a1, const __grid_constant__ CUtensorMap tmap_b1,
                        const __grid_constant__ CUtensorMap tmap_c0, const __grid_constant__ CUtensorMap tmap_c1,
                        const __grid_constant__ SliceSchedule sched, const __grid_constant__ TcParams prm) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + P2_STAGES * P2_STAGE_BYTES);
  uint64_t* empty = full + P2_STAGES;
  uint64_t* tfull = empty + P2_STAGES;
  uint64_t* tempty = tfull + 2;
  uint64_t* drain = tempty + 2;
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(drain + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_holder + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t rank = cluster_ctarank();
  const bool leader = (rank == 0);
  const int cluster = blockIdx.x >> 1, nclusters = gridDim.x >> 1;
  const int ntiles = prm.total_tiles;   // pair tiles
  const int G = prm.dev_ngroups ? *prm.dev_ngroups : sched.ngroups;   // CRT: the device plan's moduli
  const int nunits = (EPI == TC_EPI_CRT) ? ntiles * G : ntiles;

  if (threadIdx.x == 0) {
    for (int i = 0; i < P2_STAGES; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&tfull[i], 1);
      mbar_init(&tempty[i], 2 * P2Shape<EPI>::EPI_WARPS);   // one arrival per epilogue warp of both CTAs
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
    tmem_alloc_pair(tmem_holder, P2_TMEM_COLS);
    tmem_relinquish_pair();
  }
  tc_fence_before();
  cluster_sync_all();   // barriers of both CTAs initialised, TMEM allocated pair-wide
  tc_fence_after();
  const uint32_t tmem_base = *tmem_holder;
  // the leader's barriers, as seen from either CTA
  const uint32_t full_leader0 = mapa_shared(smem_u32(&full[0]), 0);
  const uint32_t tempty_leader0 = mapa_shared(smem_u32(&tempty[0]), 0);

  if (warp == 0) {
    // ------------------------------------------------------------ TMA producer (both CTAs)
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      int issued_parity[P2_STAGES];
      for (int i = 0; i < P2_STAGES; ++i) issued_parity[i] = -1;
      bool ok = true;
      for (int u = cluster; u < nunits && ok; u += nclusters) {
        int t, g0, g1;
        p2_unit<EPI>(u, ntiles, G, t, g0, g1);
        const int pr = p2_problem_of(prm, t);
        const TcProblem& P = prm.prob[pr];
        const CUtensorMap* ta = pr ? &tmap_a1 : &tmap_a0;
        const CUtensorMap* tb = pr ? &tmap_b1 : &tmap_b0;
        int tm, tn;
        p2_tile_coords(t - P.tile_begin, P.tiles_m, P.tiles_n, prm.band, tm, tn);
        const int m0 = tm * 256 + 128 * static_cast<int>(rank);
        const int n0 = tn * 256 + 128 * static_cast<int>(rank);
        for (int g = g0; g < g1 && ok; ++g) {
          for (int c = 0; c < P.nchunks && ok; ++c) {
            const int kb0 = c * sched.kb_chunk;
            const int kb1 = min(kb0 + sched.kb_chunk, P.kb_total);
            for (int i = 0; i < sched.npairs[g] && ok; ++i) {
              const int pa = sched.pp[sched.pair_off[g] + i];
              const int pb = sched.pq[sched.pair_off[g] + i];
              for (int kb = kb0; kb < kb1; ++kb) {
                if (!mbar_wait_bounded(&empty[stage], phase ^ 1, prm.wait_limit_ns, abort_flag, prm.status, 1)) {
                  ok = false;
                  break;
                }
                uint8_t* sa = smem + stage * P2_STAGE_BYTES;
                uint8_t* sb = sa + P2_A_BYTES;
                const uint32_t fbar = full_leader0 + static_cast<uint32_t>(stage) * 8u;
                if (leader) mbar_arrive_expect_tx(&full[stage], 2 * P2_STAGE_BYTES);   // both CTAs' bytes
                tma_load_3d_pair(sa, ta, fbar, kb * TC_BK, m0, pa);
                tma_load_3d_pair(sb, tb, fbar, kb * TC_BK, n0, pb);
                issued_parity[stage] = static_cast<int>(phase);
                if (++stage == P2_STAGES) { stage = 0; phase ^= 1; }
              }
            }
          }
        }
      }
      if (!ok) {
        if (leader) {
          for (int i = 0; i < P2_STAGES; ++i)
            if (issued_parity[i] >= 0) {
              volatile int no_abort = 0;
              mbar_wait_bounded(&full[i], static_cast<uint32_t>(issued_parity[i]), P2_CLEANUP_WAIT_NS, &no_abort,
                                nullptr, 0);
            }
        } else {
          // copies of this CTA are counted on the leader's barriers: give them time to land
          for (int i = 0; i < 100; ++i) __nanosleep(1000);
        }
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer (leader only)
    if (lane == 0 && leader) {
      constexpr uint32_t IDESC = idesc_bf16_f32(256, 256);
      int stage = 0;
      uint32_t phase = 0;
      int buf = 0;
      uint32_t acc_phase = 0;
      bool ok = true;
      bool issued_any = false;
      for (int u = cluster; u < nunits && ok; u += nclusters) {
        int t, g0, g1;
        p2_unit<EPI>(u, ntiles, G, t, g0, g1);
        const TcProblem& P = prm.prob[p2_problem_of(prm, t)];
        for (int g = g0; g < g1 && ok; ++g) {
          for (int c = 0; c < P.nchunks && ok; ++c) {
            const int kb0 = c * sched.kb_chunk;
            const int kb1 = min(kb0 + sched.kb_chunk, P.kb_total);
            if (!mbar_wait_bounded(&tempty[buf], acc_phase ^ 1, prm.wait_limit_ns, abort_flag, prm.status, 2)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t d_tmem = tmem_base + static_cast<uint32_t>(buf * TC_BN);
            // CRT: chunk c accumulates onto the residue of chunk c - 2, which the epilogue
            // stored back into this buffer
            uint32_t accumulate = (EPI == TC_EPI_CRT && c >= 2) ? 1u : 0u;
            for (int i = 0; i < sched.npairs[g] && ok; ++i) {
              for (int kb = kb0; kb < kb1; ++kb) {
                if (!mbar_wait_bounded(&full[stage], phase, prm.wait_limit_ns, abort_flag, prm.status, 3)) {
                  ok = false;
                  break;
                }
                tc_fence_after();
                const uint32_t sa = smem_u32(smem + stage * P2_STAGE_BYTES);
                const uint32_t sb = sa + P2_A_BYTES;
                const uint64_t adesc = smem_desc_sw128(sa);
                const uint64_t bdesc = smem_desc_sw128(sb);
#pragma unroll
                for (int kk = 0; kk < TC_BK / 16; ++kk) {
                  tc_mma_f16_pair(d_tmem, adesc + static_cast<uint64_t>(kk * 2), bdesc + static_cast<uint64_t>(kk * 2),
                                  IDESC, accumulate);
                  accumulate = 1;
                }
                issued_any = true;
                tc_commit_pair_multicast(&empty[stage], 0x3);   // frees the stage in both CTAs
                if (++stage == P2_STAGES) { stage = 0; phase ^= 1; }
              }
            }
            if (!ok) break;
            tc_commit_pair_multicast(&tfull[buf], 0x3);       // both CTAs' epilogues may drain
            if (++buf == 2) { buf = 0; acc_phase ^= 1; }
          }
        }
      }
      if (!ok && issued_any) {
        tc_commit_pair(drain);
        volatile int no_abort = 0;
        mbar_wait_bounded(drain, 0, P2_CLEANUP_WAIT_NS, &no_abort, nullptr, 0);
      }
    }
  } else {
    // ------------------------------------------------------------ epilogue (both CTAs)
    const int q = warp & 3;
    const int row_l = q * 32 + lane;
    constexpr int COLS = P2Shape<EPI>::COLS;
    const int col0 = ((warp - 2) >> 2) * COLS;
    const uint64_t keep = l2_policy_evict_last();
    int buf = 0;
    uint32_t acc_phase = 0;
    bool ok = true;
    for (int u = cluster; u < nunits && ok; u += nclusters) {
      int t, g0, g1;
      p2_unit<EPI>(u, ntiles, G, t, g0, g1);
      const int pr = p2_problem_of(prm, t);
      const TcProblem& P = prm.prob[pr];
      int tm, tn;
      p2_tile_coords(t - P.tile_begin, P.tiles_m, P.tiles_n, prm.band, tm, tn);
      const int64_t row = static_cast<int64_t>(tm) * 256 + 128 * static_cast<int>(rank) + row_l;
      const int64_t n0 = static_cast<int64_t>(tn) * 256;
      const bool row_ok = row < P.M;
      const double alpha = P.alpha, beta = P.beta;
      int ea = 0;
      if (EPI == TC_EPI_OZAKI_F64) ea = row_ok ? P.ea[row] : 0;
      double* __restrict__ tws = prm.tws ? prm.tws + static_cast<int64_t>(blockIdx.x) * (TC_BM * TC_BN) : nullptr;
      int step = 0;
      const int nsteps = G * P.nchunks;
      uint32_t racc[EPI == TC_EPI_CRT ? COLS / 4 : 1];   // CRT: running residues, 4 bytes per register
      for (int g = g0; g < g1 && ok; ++g) {
        const int wexp = 2 - sched.level[g] * sched.bits;
        const unsigned long long wbias = static_cast<unsigned long long>(896 + wexp) << 23;
        for (int c = 0; c < P.nchunks; ++c, ++step) {
          ok = __all_sync(0xffffffffu,
                          mbar_wait_bounded(&tfull[buf], acc_phase, prm.wait_limit_ns, abort_flag, prm.status, 4));
          if (!ok) break;
          tc_fence_after();
          const bool first = (step == 0), last = (step == nsteps - 1);
          const uint32_t taddr = tmem_base + (static_cast<uint32_t>(q * 32) << 16) + static_cast<uint32_t>(buf * TC_BN);
          if (EPI == TC_EPI_CRT) {
            // Chunk c of modulus p holds D = S_c + r_{c-2} (the MMA accumulated onto the residue
            // the drain of chunk c - 2 stored back into this buffer; S_c is the exact integer
            // chunk sum, |D| <= 1024 * 127^2 + 127 < 2^24, exact in FP32).  One reduction
            // r_c = D - p * rint(D / p) gives |r_c| <= 127 since p <= 253, and r_c goes back to
            // TMEM for chunk c + 2.  The two chains (even and odd chunks) meet at the end: the
            // drain of chunk nc - 2 keeps its residue in registers (biased bytes r + 128), the
            // last drain adds it, multiplies by the reconstruction's psi (mod p) and writes the
            // biased bytes to the residue plane (rows and columns padded to whole tiles, so
            // always in bounds).
            constexpr float MAGIC = 12582912.0f;   // 1.5 * 2^23: x + MAGIC - MAGIC = rint(x), |x| < 2^22
            constexpr float BIAS_F = 8388736.0f;   // 2^23 + 128: the low byte of (r + BIAS_F) is r + 128
            const float pf = prm.crt_p[g], inv = prm.crt_inv[g], psi = prm.crt_psi[G - 1][g];
            const int nc = P.nchunks;
            const bool to_tmem = (c + 2 < nc), final_c = (c == nc - 1);
            const int64_t ld = prm.res_ld;
#pragma unroll
            for (int bi = 0; bi < COLS / 16; ++bi) {   // 16 columns per TMEM load
              uint32_t v[16];
              tmem_ld_32x32b_x16(taddr + col0 + bi * 16, v);
              tc_wait_ld();
#pragma unroll
              for (int j = 0; j < 16; ++j) {
                const float d = __uint_as_float(v[j]);
                const float q = fmaf(d, inv, MAGIC) - MAGIC;
                v[j] = __float_as_uint(fmaf(-pf, q, d));
              }
              if (to_tmem) {
                tmem_st_32x32b_x16(taddr + col0 + bi * 16, v);
              } else {
#pragma unroll
                for (int j4 = 0; j4 < 4; ++j4) {
                  uint32_t rb[4];
#pragma unroll
                  for (int jj = 0; jj < 4; ++jj) {
                    float r = __uint_as_float(v[j4 * 4 + jj]);
                    if (final_c) {
                      if (nc >= 2) {
                        // add the other chain's residue (0x4B0000bb as a float is 2^23 + bb)
                        const float t = r + (__uint_as_float(__byte_perm(racc[bi * 4 + j4], 0x4B000000u, 0x7540u + jj)) - BIAS_F);
                        const float q = fmaf(t, inv, MAGIC) - MAGIC;
                        r = fmaf(-pf, q, t);
                      }
                      // times the reconstruction multiplier psi (|r psi| <= 127 * 252, exact)
                      const float t2 = r * psi;
                      const float q2 = fmaf(t2, inv, MAGIC) - MAGIC;
                      r = fmaf(-pf, q2, t2);
                    }
                    rb[jj] = __float_as_uint(r + BIAS_F);
                  }
                  racc[bi * 4 + j4] =
                      __byte_perm(__byte_perm(rb[0], rb[1], 0x0040u), __byte_perm(rb[2], rb[3], 0x0040u), 0x5410u);
                }
              }
            }
            if (to_tmem) tc_wait_st();
            if (final_c) {
              uint8_t* __restrict__ dst = prm.res + g * prm.res_plane + (n0 + col0) * ld + row;
#pragma unroll
              for (int w = 0; w < COLS / 4; ++w) {
#pragma unroll
                for (int jj = 0; jj < 4; ++jj) {
                  *dst = static_cast<uint8_t>(racc[w] >> (8 * jj));
                  dst += ld;
                }
              }
            }
          } else
#pragma unroll 1
          for (int cb = col0; cb < col0 + COLS; cb += 32) {
            uint32_t v[32];
            tmem_ld_32x32b_x32(taddr + cb, v);
            tc_wait_ld();
            const int64_t colb = n0 + cb;
            if (EPI == TC_EPI_F32) {
              if (prm.c_tma && beta == 0.0 && row - lane + 32 <= P.M && colb + 32 <= P.N) {
                // C through shared memory and a TMA store of the warp's 32 x 32 box; boxes that
                // reach past C's last row or column take the direct stores below (measured: a
                // store box that crosses the last row was not clipped at the row but at the next
                // 16-byte boundary, writing rows of the caller's padding).  The box buffer is
                // reused once the previous store of this warp has read it.
                float* cbuf = reinterpret_cast<float*>(smem + P2_CSTAGE_OFF + (warp - 2) * 4096);
                const float fa = static_cast<float>(alpha);
                if (lane == 0) bulk_wait_read_all();
                __syncwarp();
#pragma unroll
                for (int j = 0; j < 32; ++j) cbuf[j * 32 + lane] = fa * __uint_as_float(v[j]);
                fence_proxy_async_smem();
                __syncwarp();
                if (lane == 0) {
                  tma_store_2d(pr ? &tmap_c1 : &tmap_c0, cbuf, static_cast<int>(row - lane), static_cast<int>(colb));
                  bulk_commit_group();
                }
                continue;
              }
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
            double tv[32];
            if (!first) {
#pragma unroll
              for (int j = 0; j < 32; ++j) tv[j] = ld_f64_hint(tcol + j * TC_BM, keep);
            }
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              const double sw = p2_exact_int_f32_times_pow2(v[j], wbias);
              tv[j] = first ? sw : tv[j] + sw;
            }
            if (!last) {
#pragma unroll
              for (int j = 0; j < 32; ++j) st_f64_hint(tcol + j * TC_BM, tv[j], keep);
            } else if (row_ok) {
              double* __restrict__ crow = static_cast<double*>(P.C) + row + colb * P.ldc;
#pragma unroll
              for (int j8 = 0; j8 < 32; j8 += 8) {
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
                  if (ea == P2_EXP_NONFINITE || ebj[j] == P2_EXP_NONFINITE)
                    val = __longlong_as_double(0x7FF8000000000000ll);
                  else
                    val = scale_pow2(tv[j8 + j], ea + ebj[j]);
                  crow[(j8 + j) * P.ldc] = (beta == 0.0) ? alpha * val : fma(alpha, val, beta * c0[j]);
                }
              }
            }
          }
          // the whole warp has drained its columns: one arrival on the leader's tmem_empty
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive_cluster(tempty_leader0 + static_cast<uint32_t>(buf) * 8u);
          if (++buf == 2) { buf = 0; acc_phase ^= 1; }
        }
      }
    }
  }

  if (EPI == TC_EPI_F32 && prm.c_tma && warp >= 2 && lane == 0) bulk_wait_all();   // C stores done
  tc_fence_before();
  __syncthreads();
  cluster_sync_all();   // neither CTA releases TMEM or exits while its peer still works
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    tmem_dealloc_pair(tmem_base, P2_TMEM_COLS);
  }
}

int tc_gemm_pair_launch(int epi, const CUtensorMap& ta0, const CUtensorMap& tb0, const CUtensorMap* ta1,
                        const CUtensorMap* tb1, const SliceSchedule& sched, const TcParams& prm, int grid,
                        int kernel_kind, cudaStream_t s, const CUtensorMap* tc0, const CUtensorMap* tc1) {
  static std::atomic<unsigned long long> smem_opt_in[3];   // per kernel, one bit per device
  const CUtensorMap& a1 = ta1 ? *ta1 : ta0;
  const CUtensorMap& b1 = tb1 ? *tb1 : tb0;
  // C maps are read only when prm.c_tma is set (TC_EPI_F32); otherwise any map fills the slots
  const CUtensorMap& c0 = tc0 ? *tc0 : ta0;
  const CUtensorMap& c1 = tc1 ? *tc1 : c0;
  if (prm.c_tma && (epi != TC_EPI_F32 || !tc0 || (prm.nprob == 2 && !tc1))) return GB_ERR_INVALID_VALUE;
  if (grid < 2) grid = 2;
  grid &= ~1;
  if (epi == TC_EPI_OZAKI_F64) {
    const int rc = opt_in_dynamic_smem(tc_gemm_pair_kernel<TC_EPI_OZAKI_F64>, P2_SMEM_BYTES, smem_opt_in[0]);
    if (rc) return rc;
    GB_LAUNCH(kernel_kind, s,
              (tc_gemm_pair_kernel<TC_EPI_OZAKI_F64><<<grid, P2Shape<TC_EPI_OZAKI_F64>::THREADS, P2_SMEM_BYTES, s>>>(ta0, tb0, a1, b1, c0, c1, sched, prm)));
  } else if (epi == TC_EPI_CRT) {
    const int rc = opt_in_dynamic_smem(tc_gemm_pair_kernel<TC_EPI_CRT>, P2_SMEM_BYTES, smem_opt_in[2]);
    if (rc) return rc;
    GB_LAUNCH(kernel_kind, s,
              (tc_gemm_pair_kernel<TC_EPI_CRT><<<grid, P2Shape<TC_EPI_CRT>::THREADS, P2_SMEM_BYTES, s>>>(ta0, tb0, a1, b1, c0, c1, sched, prm)));
  } else {
    const int rc = opt_in_dynamic_smem(tc_gemm_pair_kernel<TC_EPI_F32>, P2_SMEM_BYTES_F32, smem_opt_in[1]);
    if (rc) return rc;
    GB_LAUNCH(kernel_kind, s,
              (tc_gemm_pair_kernel<TC_EPI_F32><<<grid, P2Shape<TC_EPI_F32>::THREADS, P2_SMEM_BYTES_F32, s>>>(ta0, tb0, a1, b1, c0, c1, sched, prm)));
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

}  // namespace gb
