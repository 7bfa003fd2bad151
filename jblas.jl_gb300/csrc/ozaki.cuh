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

// Per-row statistics of op(X) (rows r < R, contraction index k < K), cut into `kslices`
// K slices: amax bits of |x| per row (uint64, exact; zeroed and filled by oz_row_stats),
// and per slice s the exponent e_s of the slice's max (max < 2^e_s) with FP32 sums of
// |x| 2^-e_s and x^2 2^-2e_s over truncated values ([s][R] arrays; only with sums = true).
// The host rescales the slice sums to the row exponent and bounds them one-sidedly.
struct OzRowStats {
  unsigned long long* amax_bits;
  int32_t* part_e;
  float* part_sa;
  float* part_sq;
  int32_t kslices;
};

// K slices the statistics kernel uses for this layout (1 when k is contiguous).
int oz_stats_kslices(int64_t R, int64_t K, int64_t ks, int sms);
int oz_row_stats(const double* X, int64_t R, int64_t K, int64_t rs, int64_t ks, OzRowStats st, bool sums,
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
  int engine;             // 1 = one CTA per 128 x 256 tile, 2 = CTA pairs on 256 x 256 tiles
  int band;               // tile rows per L2 band of the raster
};
int oz_gemm_launch(const OzGemmArgs& a, const OzPlan& plan, cudaStream_t s);
// Persistent grid size: one CTA per SM, at most one per output tile.
int oz_grid_for(int sms, int64_t M, int64_t N, int engine);

// ---------------------------------------------------------------- CRT mode (ozaki_crt.cu)
// Constants of the CRT mode, fixed by the moduli table; passed by value to the kernels.
struct CrtModuli {                  // per modulus g (independent of how many a call uses)
  uint32_t p[TC_MAX_MODULI];        // the moduli (pairwise coprime, <= 253)
  float climb4[TC_MAX_MODULI][3];   // split, t <= 52: 2^(14 (l + 1)) mod p in (-p/2, p/2], l = 0..2
  float climb5[TC_MAX_MODULI][4];   // split, t > 52: 2^(13 (l + 1)) mod p, l = 0..3
  float pf[TC_MAX_MODULI];          // p as a float
  float pinv[TC_MAX_MODULI];        // fl32(1 / p)
};
// Reconstruction with the first n moduli, M = their product.  The moduli are taken in
// groups of up to three consecutive ones (P_G = their product < 2^24); the residue planes
// hold x_g = psi_G C' mod p_g (psi_G = (M / P_G)^-1 mod P_G, applied in the last drain of
// the residue products), so that v_G = CRT_G(x) = psi_G C' mod P_G and
// C' = sum_G v_G (M / P_G) - k M.
constexpr int CRT_MAX_GROUPS = (TC_MAX_MODULI + 2) / 3;
struct CrtRecon {
  int32_t ngroups;
  int32_t pad;
  float psi[TC_MAX_MODULI];         // psi_G mod p_g for the group G holding modulus g
  float a1[CRT_MAX_GROUPS];         // (p_a)^-1 mod p_b          (group moduli a, b, c)
  float pa[CRT_MAX_GROUPS];         // p_a
  float a2[CRT_MAX_GROUPS];         // (p_a p_b)^-1 mod p_c
  float pab[CRT_MAX_GROUPS];        // p_a p_b
  float P[CRT_MAX_GROUPS];          // P_G
  float Pinv[CRT_MAX_GROUPS];       // fl32(1 / P_G)
  int32_t voff[CRT_MAX_GROUPS];     // P_G - (2^23 + 128): biased group value -> v + P_G
  float ks0;                        // fl32(sum_G (P_G - 2^23 - 128) / P_G)
  uint32_t w[CRT_MAX_GROUPS][4];    // M / P_G mod 2^128, little-endian 32-bit words
  uint32_t m[4];                    // M mod 2^128
};
struct CrtTable {
  CrtModuli mod;
  CrtRecon rec[TC_MAX_MODULI];      // rec[n - 1]: the first n moduli
};

// The plan of one CRT call, written on the device by the planner kernel (no host round trip)
// into the call's own workspace and read by the split, residue-product and combine kernels.
struct CrtDevicePlan {
  int32_t n;        // moduli
  int32_t t;        // integer bits of the scaled operands
  double bound;     // a-priori normwise error bound of the plan
};
// A copy of a call's plan for reading back on the host (gb_last_ozaki_plan), tagged with the
// call's sequence number; kept in a per-device ring that no kernel reads.
struct CrtPlanRecord {
  CrtDevicePlan plan;
  unsigned long long seq;
};

// Inputs of the planner besides the statistics.
struct CrtPlanParams {
  int64_t M, N, K;
  int32_t n_fixed;                      // > 0: this many moduli with t = t_fixed
  int32_t t_fixed;
  int32_t with_sums;                    // the statistics carry K-slice sums (else no bound)
  int32_t pad;
  double tol;                           // normwise tolerance for the automatic choice
  double log2m[TC_MAX_MODULI + 1];      // log2 of the product of the first n moduli
  int32_t tk[TC_MAX_MODULI + 1];        // crt_bits_for(K, n), used when statistics are not finite
};

struct CrtPlan {
  int n, t;
  int64_t k_chunk;
  int32_t kb_total;
  int nchunks;
  double flops_tensor;
  double log2_m;
  SliceSchedule sched;   // one group per modulus, pair (g, g)
};

const uint32_t* crt_moduli();       // TC_MAX_MODULI moduli, in the order they are used
double crt_log2_product(int n);     // log2 of the product of the first n moduli
// Largest t <= 62 with 4 K 2^(2t) <= prod(first n moduli) and K 2^(2t) <= 2^125 (0: none).
int crt_bits_for(int64_t K, int n);
// Plan for n moduli and t integer bits (t = 0: crt_bits_for(K, n)).
int crt_make_plan(int64_t M, int64_t N, int64_t K, int n, int t, CrtPlan* plan);
// The constant table (built once on the host).
const CrtTable& crt_table();
// A read-back record from the current device's ring (reused after CRT_PLAN_RING calls; the
// record's tag tells whether it still holds the call `seq`).
constexpr int CRT_PLAN_RING = 4096;
int crt_plan_record(CrtPlanRecord** record, unsigned long long* seq);
// Planner: from the statistics (with sums), the fewest moduli whose bound meets pp.tol (or
// pp.n_fixed) and the widest t they allow; writes *plan (the call's workspace) and the tagged
// copy *record on the device.  `scratch` holds crt_plan_scratch_bytes() bytes of stream-ordered
// workspace.
size_t crt_plan_scratch_bytes();
int crt_plan_device(const OzRowStats& sa, const OzRowStats& sb, const CrtPlanParams& pp, CrtDevicePlan* plan,
                    CrtPlanRecord* record, unsigned long long seq, void* scratch, cudaStream_t s);
// Residue planes (BF16, [modulus][row][pitch], plan->n of them) and row exponents of rows
// [0, R) of op(X); the planes belong to an operand of plane_rows >= R rows (a band of rows
// passes X, amax_bits, planes and exps offset to its first row, and the operand's row count).
int crt_split(const double* X, int64_t R, int64_t K, int64_t rs, int64_t ks, const unsigned long long* amax_bits,
              const CrtDevicePlan* plan, __nv_bfloat16* planes, int64_t pitch, int64_t plane_rows, int32_t* exps,
              cudaStream_t s);

struct CrtGemmArgs {
  const void* planes_a;   // [n][M][pitch] bf16
  const void* planes_b;   // [n][N][pitch] bf16
  int64_t pitch;
  int64_t M, N, K;
  const int32_t* ea;
  const int32_t* eb;
  double alpha, beta;
  double* C;
  int64_t ldc;
  uint8_t* res;           // [n][ceil(N/256)*256][res_ld] residues, biased bytes r + 128
  int64_t res_ld;         // ceil(M/256)*256
  int64_t res_plane;
  DeviceStatus* status;
  uint64_t wait_limit_ns;
  int grid;               // even (CTA pairs)
  const CrtDevicePlan* plan;
  int band;               // pair-tile rows per L2 band of the raster
  int64_t a_plane_rows;   // rows of the operands whose planes planes_a / planes_b point into
  int64_t b_plane_rows;   // (>= M, N; a block of C passes both at its first row / column)
};
// Residue products on the CTA-pair engine (crt_mma_launch), then the CRT reconstruction into C
// (crt_combine_launch).  `plan` (host) gives the K chunking and a schedule for up to plan.n
// moduli; the kernels run the device plan's n <= plan.n.  A block of C passes planes_a, ea,
// planes_b, eb, C and res offset to its first row and column (multiples of 256) and M, N = its
// size.
int crt_mma_launch(const CrtGemmArgs& a, const CrtPlan& plan, cudaStream_t s);
int crt_combine_launch(const CrtGemmArgs& a, cudaStream_t s);


}  // namespace gb
