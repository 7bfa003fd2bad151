// FP32 GEMM on the BF16 tensor cores by term splitting: C = alpha op(A) op(B) + beta C.
//
// No reference counterpart as an algorithm: jBLAS's Float32 jmul! (src/gemm.jl:244) is an FMA
// chain, which the NATIVE mode of gb_gemm_f32 reproduces bit for bit on the CUDA cores.  This
// mode trades that bit-exactness for the tensor cores.  Every FP32 value is split into BF16
// terms x = t_0 + t_1 (+ t_2) (split_bf16_terms, adjoint.cu) and the product keeps the term
// pairs (p, q) with p + q below the term count:
//   BF16X3: 2 terms, pairs (0,0), (0,1), (1,0)                 |dropped| <= 2^-16 |x y|
//   BF16X6: 3 terms, pairs (0,0), (0,1), (1,0), (0,2), (1,1), (2,0)
//                                                              |dropped| <= 2^-23 |x y|
// all accumulated in one FP32 TMEM accumulator per output tile by the slice-product engine
// (tc_gemm2.cu / tc_gemm.cu, TC_EPI_F32 epilogue with alpha and beta).  Per element the error is
// at most about (2^-15 + K 2^-24) (|op(A)| |op(B)|)_ij for BF16X3 and (2^-21 + K 2^-24) (...)_ij
// for BF16X6 (FP32 accumulation of K terms).
//
// Operand planes, K-major BF16 as the engine reads them: op(A) as [term][i][k] and op(B) as
// [term][j][k], pitch = K rounded up to 64.
#include <cuda_bf16.h>

#include <cstring>

#include "gb_common.cuh"
#include "profile.cuh"
#include "tc_gemm.cuh"

namespace gb {

int split_bf16_terms(const float* X, int64_t R, int64_t Kd, int64_t rs, int64_t ks, int nterms,
                     __nv_bfloat16* planes, int64_t pitch, __nv_bfloat16* planes_t, int64_t pitch_t, int kind,
                     cudaStream_t s);

static inline int64_t pitch64_of(int64_t k) { return ((k + 63) / 64) * 64; }
static inline size_t align_256(size_t x) { return (x + 255) & ~size_t(255); }

size_t gemm_f32_tc_workspace_bytes(int64_t M, int64_t N, int64_t K, int nterms) {
  const size_t pk = static_cast<size_t>(pitch64_of(K));
  return align_256(static_cast<size_t>(nterms) * M * pk * 2) + align_256(static_cast<size_t>(nterms) * N * pk * 2);
}

// One group holding the kept term pairs, smallest contributions first.
static void term_schedule(SliceSchedule& S, int nterms, int kb_chunk) {
  std::memset(&S, 0, sizeof(S));
  S.ngroups = 1;
  S.kb_chunk = kb_chunk;
  S.level[0] = 0;
  S.pair_off[0] = 0;
  int n = 0;
  for (int level = nterms - 1; level >= 0; --level)
    for (int p = 0; p <= level; ++p) {
      S.pp[n] = static_cast<uint8_t>(p);
      S.pq[n] = static_cast<uint8_t>(level - p);
      ++n;
    }
  S.npairs[0] = static_cast<int8_t>(n);
}

int gemm_f32_tc(int ta, int tb, int64_t M, int64_t N, int64_t K, float alpha, const float* A, int64_t lda,
                const float* B, int64_t ldb, float beta, float* C, int64_t ldc, int nterms, void* ws, int sms,
                DeviceStatus* status, uint64_t wait_limit_ns, cudaStream_t s) {
  const int64_t pk = pitch64_of(K);
  __nv_bfloat16* PA = static_cast<__nv_bfloat16*>(ws);
  __nv_bfloat16* PB = reinterpret_cast<__nv_bfloat16*>(static_cast<char*>(ws) +
                                                       align_256(static_cast<size_t>(nterms) * M * pk * 2));
  // op(A)[i, k] = ta ? A[k + i lda] : A[i + k lda];  op(B)[k, j] = tb ? B[j + k ldb] : B[k + j ldb]
  int rc = split_bf16_terms(A, M, K, ta ? lda : 1, ta ? 1 : lda, nterms, PA, pk, nullptr, 0, GB_KERNEL_F32_SPLIT, s);
  if (!rc)
    rc = split_bf16_terms(B, N, K, tb ? 1 : ldb, tb ? ldb : 1, nterms, PB, pk, nullptr, 0, GB_KERNEL_F32_SPLIT, s);
  if (rc) return rc;
  const TcTuning tune = tc_tuning_for(TC_KIND_F32, M, N);
  const bool pair = tune.engine == 2;
  CUtensorMap tmap_a, tmap_b;
  rc = make_plane_tmap(&tmap_a, PA, K, M, nterms, pk, TC_BM);
  if (!rc) rc = make_plane_tmap(&tmap_b, PB, K, N, nterms, pk, pair ? 128 : TC_BN);
  if (rc) return rc;
  const int64_t tbm = pair ? 256 : TC_BM, tbn = pair ? 256 : TC_BN;
  TcParams prm;
  std::memset(&prm, 0, sizeof(prm));
  prm.band = tune.band;
  TcProblem& P = prm.prob[0];
  P.M = M;
  P.N = N;
  P.K = K;
  P.tiles_m = static_cast<int32_t>((M + tbm - 1) / tbm);
  P.tiles_n = static_cast<int32_t>((N + tbn - 1) / tbn);
  P.tile_begin = 0;
  P.kb_total = static_cast<int32_t>((K + TC_BK - 1) / TC_BK);
  P.nchunks = 1;
  P.C = C;
  P.ldc = ldc;
  P.alpha = alpha;
  P.beta = beta;
  prm.nprob = 1;
  prm.total_tiles = P.tiles_m * P.tiles_n;
  prm.status = status;
  prm.wait_limit_ns = wait_limit_ns;
  SliceSchedule sched;
  term_schedule(sched, nterms, P.kb_total);
  if (pair) {
    CUtensorMap tmap_c;
    prm.c_tma = (tune.tma_store && beta == 0.0f && make_c_tmap_f32(&tmap_c, C, M, N, ldc)) ? 1 : 0;
    const int64_t ctas = 2 * static_cast<int64_t>(prm.total_tiles), cap = sms & ~1;
    return tc_gemm_pair_launch(TC_EPI_F32, tmap_a, tmap_b, nullptr, nullptr, sched, prm,
                               static_cast<int>(ctas < cap ? ctas : cap), GB_KERNEL_F32_MMA, s,
                               prm.c_tma ? &tmap_c : nullptr, nullptr);
  }
  const int grid = prm.total_tiles < sms ? prm.total_tiles : sms;
  return tc_gemm_launch(TC_EPI_F32, tmap_a, tmap_b, nullptr, nullptr, sched, prm, grid, GB_KERNEL_F32_MMA, s);
}

}  // namespace gb
