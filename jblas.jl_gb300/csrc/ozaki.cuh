// Ozaki-scheme FP64 emulation on BF16 tensor cores: planner structures and launchers.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "gb_common.cuh"
#include "tc_gemm.cuh"

namespace gb {

constexpr int OZ_MAX_SLICES = 20;

// Host-side plan of one Ozaki product.
struct OzPlan {
  int slices;
  int bits;
  int64_t k_chunk;
  int32_t kb_total;
  int products;   // pairs with p + q <= slices + 1
  int groups;     // TMEM groups per K chunk
  int nchunks;
  double flops_tensor;
  SliceSchedule sched;
};

// bits per digit plane for an exact FP32 sum of `kc` products of `pairs_per_group` pairs.
int oz_bits_for(int64_t kc);
// Builds the plan (schedule included) for a given slice count (1..OZ_MAX_SLICES).
int oz_make_plan(int64_t M, int64_t N, int64_t K, int slices, OzPlan* plan);
// Same, with K cut into at least `min_chunks` exact accumulation chunks (wider digits).
int oz_make_plan_chunks(int64_t M, int64_t N, int64_t K, int slices, int min_chunks, OzPlan* plan);
// Relative per-tile cost of a plan (tensor work vs FP64 drains), for choosing among plans.
double oz_plan_cost(const OzPlan& p);

// Per-row statistics of op(X) (rows r < R, contraction index k < K): amax bits of |x|
// (as uint64, exact), and FP32 sums of |x| 2^-e and x^2 2^-2e over truncated values, e the
// row exponent (max |x| < 2^e); the host turns them into one-sided bounds.
struct OzRowStats {
  unsigned long long* amax_bits;
  double* sum_abs;
  double* sum_sq;
};

int oz_row_stats(const double* X, int64_t R, int64_t K, int64_t rs, int64_t ks, OzRowStats st,
                 cudaStream_t s);
// Writes `slices` digit planes (BF16, [slice][row][pitch]) and per-row exponents.
int oz_split(const double* X, int64_t R, int64_t K, int64_t rs, int64_t ks,
             const unsigned long long* amax_bits, int slices, int bits, __nv_bfloat16* planes,
             int64_t pitch, int32_t* exps, cudaStream_t s);

struct OzGemmArgs {
  const void* planes_a;   // [slices][M][pitch] bf16
  const void* planes_b;   // [slices][N][pitch] bf16
  int64_t pitch;          // elements per plane row (multiple of 64)
  int slices;
  int64_t M, N, K;
  const int32_t* ea;      // row exponents of op(A)
  const int32_t* eb;      // column exponents of op(B)
  double alpha, beta;
  double* C;
  int64_t ldc;
  double* tws;            // per-CTA FP64 tile buffers (grid x 128 x 256)
  DeviceStatus* status;
  uint64_t wait_limit_ns;
  int grid;
};
int oz_gemm_launch(const OzGemmArgs& a, const OzPlan& plan, cudaStream_t s);
// Persistent grid size: one CTA per SM, at most one per output tile.
int oz_grid_for(int sms, int64_t M, int64_t N);


}  // namespace gb
