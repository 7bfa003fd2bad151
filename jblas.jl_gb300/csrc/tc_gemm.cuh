// Slice-product GEMM engine on tcgen05 (BF16 operands, FP32 accumulation in TMEM).
//
// Operands are stacks of BF16 planes, K-major: plane[p][row][k] with a row pitch that is
// a multiple of 64 elements.  A schedule lists groups of plane pairs (p, q); each group is
// summed into one TMEM accumulator per K chunk and handed to the epilogue:
//   TC_EPI_OZAKI_F64  exact integer group sums, accumulated in FP64 per tile (smallest
//                     level first), rescaled by 2^(ea_i + eb_j) with alpha/beta, FP64 out
//   TC_EPI_F32        one group, C = alpha * sum + beta * C in FP32 (split-BF16 products)
//   TC_EPI_CRT        one group per modulus p_g <= 253: exact chunk sums accumulated mod p_g,
//                     written as biased bytes r + 128 (|r| <= 127, r = C' mod p_g) to a
//                     residue plane (CTA-pair engine only)
// One launch may carry two independent problems (the adjoint's dA and dB); CTAs walk
// the concatenated tile list.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "gb_common.cuh"

namespace gb {

constexpr int TC_MAX_GROUPS = 256;
constexpr int TC_MAX_PAIRS = 256;
constexpr int TC_BM = 128;   // tile rows (TMEM lanes)
constexpr int TC_BN = 256;   // tile columns (TMEM columns per accumulator)
constexpr int TC_BK = 64;    // BF16 elements per 128-byte swizzled row
constexpr int TC_STAGES = 4;

enum TcEpilogue { TC_EPI_OZAKI_F64 = 0, TC_EPI_F32 = 1, TC_EPI_CRT = 2 };
constexpr int TC_MAX_MODULI = 20;

// Group g sums the products (pp[off+i], pq[off+i]), i < npairs[g], of level[g].
struct SliceSchedule {
  int32_t ngroups;
  int32_t kb_chunk;   // K panels of 64 per exact accumulation chunk
  int32_t bits;       // bits per digit plane (Ozaki weights 2^(2 - level*bits))
  int32_t pad;
  int8_t level[TC_MAX_GROUPS];
  int8_t npairs[TC_MAX_GROUPS];
  int16_t pair_off[TC_MAX_GROUPS];
  uint8_t pp[TC_MAX_PAIRS];
  uint8_t pq[TC_MAX_PAIRS];
};

struct TcProblem {
  int64_t M, N, K;
  int32_t tiles_m, tiles_n;
  int32_t tile_begin;   // first index of this problem in the launch's tile list
  int32_t kb_total;     // K panels of 64
  int32_t nchunks;      // ceil(kb_total / kb_chunk)
  int32_t pad;
  void* C;
  int64_t ldc;
  double alpha, beta;
  const int32_t* ea;    // Ozaki row / column exponents (TC_EPI_OZAKI_F64)
  const int32_t* eb;
};

struct TcParams {
  TcProblem prob[2];
  int32_t nprob;
  int32_t total_tiles;
  double* tws;          // per-CTA FP64 tile buffers (Ozaki, more than one drain per tile)
  DeviceStatus* status;
  uint64_t wait_limit_ns;
  // TC_EPI_CRT: residue planes res[g][col][row] (uint8, rows padded to res_ld, column
  // count padded to whole tiles) and, per modulus g (= group), p_g and fl32(1 / p_g)
  uint8_t* res;
  int64_t res_ld;
  int64_t res_plane;
  float crt_p[TC_MAX_MODULI];
  float crt_inv[TC_MAX_MODULI];
  const int32_t* dev_ngroups;   // when set, the number of schedule groups to run (read on the device)
  float crt_psi[TC_MAX_MODULI][TC_MAX_MODULI];   // [n - 1][g]: multiplier of the final residue
};

// Tensor maps for problem 0 and (optionally) problem 1; box 64 x 128 for A, 64 x 256 for B.
int tc_gemm_launch(int epi, const CUtensorMap& ta0, const CUtensorMap& tb0, const CUtensorMap* ta1,
                   const CUtensorMap* tb1, const SliceSchedule& sched, const TcParams& prm, int grid,
                   int kernel_kind, cudaStream_t s);

// CTA-pair form (tc_gemm2.cu): 256 x 256 tiles on two SMs; TcProblem tile counts and
// tile_begin are in 256 x 256 units, grid is even.
int tc_gemm_pair_launch(int epi, const CUtensorMap& ta0, const CUtensorMap& tb0, const CUtensorMap* ta1,
                        const CUtensorMap* tb1, const SliceSchedule& sched, const TcParams& prm, int grid,
                        int kernel_kind, cudaStream_t s);

// Engine selection: 0 = automatic (CTA pairs), 1 = single-CTA 128 x 256 tiles, 2 = CTA pairs.
int tc_engine_setting();
void tc_set_engine(int e);
inline bool tc_use_pair() { return tc_engine_setting() != 1; }

// 3-D BF16 tensor map {K, rows, planes} over [planes][rows][pitch], box 64 x box_rows x 1,
// 128-byte swizzle (defined in capi.cu).
int make_plane_tmap(CUtensorMap* map, const void* base, int64_t K, int64_t rows, int64_t slices,
                    int64_t pitch, int box_rows);

inline int tc_pair_tiles(int64_t M, int64_t N) {
  return static_cast<int>(((M + 255) / 256) * ((N + 255) / 256));
}

inline int tc_tiles(int64_t M, int64_t N) {
  return static_cast<int>(((M + TC_BM - 1) / TC_BM) * ((N + TC_BN - 1) / TC_BN));
}

}  // namespace gb
