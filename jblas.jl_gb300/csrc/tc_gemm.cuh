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
  int32_t band;         // output-tile rows per band of the tile raster (L2 reuse of the A rows)
  int32_t c_tma;        // TC_EPI_F32: 1 = C written by TMA stores from shared memory (beta = 0)
};

// ---------------------------------------------------------------- tuning (pick_kernel_size)
// Launch configuration of the engine per kind of product and output-size class, the
// GPU-side counterpart of jBLAS's micro-tile choice and block options
// (src/kernel_structure.jl:76-99, src/blas_options.jl:2-7): engine (1 = one CTA per 128 x 256
// tile, cta_group::1; 2 = a CTA pair per 256 x 256 tile, cta_group::2), band (output-tile rows
// of the L2 band of the tile raster) and, for FP32 outputs, TMA stores of C.
enum TcKind { TC_KIND_SLICES = 0, TC_KIND_CRT = 1, TC_KIND_F32 = 2, TC_KIND_ADJOINT = 3, TC_KINDS = 4 };
constexpr int TC_TUNE_CLASSES = 3;   // by max(M, N): <= 2048, <= 8192, larger
struct TcTuning {
  int32_t engine;
  int32_t band;
  int32_t tma_store;
  int32_t panels;   // CRT: column panels pipelined against the residue products (0/1 = one)
};
int tc_tune_class(int64_t M, int64_t N);
constexpr int TC_MAX_PANELS = 4;   // CRT column panels
TcTuning tc_default_tuning(int kind, int cls);
int tc_validate_tuning(int kind, const TcTuning& t);
// The tuning a call of this kind and output size uses (gb_set_tc_engine, when set, overrides
// the engine).
TcTuning tc_tuning_for(int kind, int64_t M, int64_t N);
int tc_set_tuning(int kind, int cls, const TcTuning* t);   // t = nullptr: the default
TcTuning tc_get_tuning(int kind, int cls);

// Tensor maps for problem 0 and (optionally) problem 1; box 64 x 128 for A, 64 x 256 for B.
int tc_gemm_launch(int epi, const CUtensorMap& ta0, const CUtensorMap& tb0, const CUtensorMap* ta1,
                   const CUtensorMap* tb1, const SliceSchedule& sched, const TcParams& prm, int grid,
                   int kernel_kind, cudaStream_t s);

// CTA-pair form (tc_gemm2.cu): 256 x 256 tiles on two SMs; TcProblem tile counts and
// tile_begin are in 256 x 256 units, grid is even.
// tc0 / tc1: FP32 C maps of problems 0 / 1 (make_c_tmap_f32), read when prm.c_tma is set.
int tc_gemm_pair_launch(int epi, const CUtensorMap& ta0, const CUtensorMap& tb0, const CUtensorMap* ta1,
                        const CUtensorMap* tb1, const SliceSchedule& sched, const TcParams& prm, int grid,
                        int kernel_kind, cudaStream_t s, const CUtensorMap* tc0 = nullptr,
                        const CUtensorMap* tc1 = nullptr);

// Engine override: 0 = the tuning's engine, 1 = single-CTA 128 x 256 tiles, 2 = CTA pairs.
int tc_engine_setting();
void tc_set_engine(int e);

// 3-D BF16 tensor map {K, rows, planes} over [planes][plane_rows][pitch] (plane_rows = 0: rows;
// a band of rows passes base at its first row and the planes' full row count), box
// 64 x box_rows x 1, 128-byte swizzle (defined in capi.cu).
int make_plane_tmap(CUtensorMap* map, const void* base, int64_t K, int64_t rows, int64_t slices,
                    int64_t pitch, int box_rows, int64_t plane_rows = 0);
// 2-D FP32 tensor map over a column-major M x N matrix C (leading dimension ldc), box 32 x 32,
// for the TMA-store epilogue (which stores only boxes lying wholly inside C).  false when C's layout does not allow one (base not 16-byte
// aligned, ldc not a multiple of 4, sizes beyond the map's range); the caller then stores directly.
bool make_c_tmap_f32(CUtensorMap* map, const void* C, int64_t M, int64_t N, int64_t ldc);

inline int tc_pair_tiles(int64_t M, int64_t N) {
  return static_cast<int>(((M + 255) / 256) * ((N + 255) / 256));
}

inline int tc_tiles(int64_t M, int64_t N) {
  return static_cast<int>(((M + TC_BM - 1) / TC_BM) * ((N + TC_BN - 1) / TC_BN));
}

}  // namespace gb
