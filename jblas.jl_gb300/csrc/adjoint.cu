// Adjoint of gemm!: dA = dC * B^T and dB = A^T * dC in ONE tcgen05 launch (FP32 in/out).
//
// No reference counterpart: this is the pullback a ChainRulesCore rrule for jBLAS's
// jmul!/gemm! (src/gemm.jl:244) returns.  Products use the 3xBF16 split: every FP32 value
// x is held as hi = bf16(x), lo = bf16(x - hi), and
//   x*y ~= hi_x*hi_y + hi_x*lo_y + lo_x*hi_y      (lo_x*lo_y, below 2^-16 |xy|, is dropped)
// accumulated in FP32 in TMEM: three plane pairs of one group of the slice-product engine.
//
// Operand planes (K-major BF16, two planes each: hi, lo):
//   dA = dC * B^T   left  dC as [p][i][j]   (transposed from column-major dC)
//                   right B  as [p][k][j]   (transposed from column-major B)
//   dB = A^T * dC   left  A  as [p][k][i]   (A's columns are already contiguous in i)
//                   right dC as [p][j][i]   (dC's columns are already contiguous in i)
// dC is read from memory once: one kernel writes both of its plane layouts.
#include <cuda_bf16.h>

#include <cstring>

#include "gb_common.cuh"
#include "profile.cuh"
#include "tc_gemm.cuh"

namespace gb {

// x = t_0 + t_1 (+ t_2) in BF16 terms: t_0 = bf16(x), t_1 = bf16(x - t_0), t_2 = bf16(x - t_0 - t_1).
// Each difference is exact in FP32 (it keeps the lower bits of x), so with three terms the sum is
// x exactly (24 = 3 x 8 significand bits, barring underflow); with two, |x - t_0 - t_1| <= 2^-17 |x|.
template <int NT>
__device__ __forceinline__ void split_terms(float x, uint32_t (&t)[NT]) {
  float r = x;
#pragma unroll
  for (int i = 0; i < NT; ++i) {
    const __nv_bfloat16 b = __float2bfloat16_rn(r);
    t[i] = static_cast<uint32_t>(__bfloat16_as_ushort(b));
    r -= __bfloat162float(b);
  }
}

// k contiguous or strided (element (r, k) at X[r*rs + k*ks]): one thread = one row r and 16
// consecutive k, neighbouring threads neighbouring k; writes the NT term planes
// [term][r][pitch], 32 bytes per plane per thread.  With ks == 1 the 16 values are read as four
// 16-byte loads when aligned.
template <int NT>
__global__ void __launch_bounds__(256) split_kc_kernel(const float* __restrict__ X, int64_t R, int64_t Kd,
                                                       int64_t rs, int64_t ks, __nv_bfloat16* __restrict__ planes,
                                                       int64_t pitch, int64_t plane) {
  const int64_t kc = static_cast<int64_t>(blockIdx.x) * 256 + threadIdx.x, r = blockIdx.y;
  const int64_t k0 = kc * 16;
  if (r >= R || k0 >= Kd) return;
  const int nvalid = static_cast<int>(Kd - k0 < 16 ? Kd - k0 : 16);
  const float* src = X + r * rs + k0 * ks;
  float x[16];
  if (ks == 1 && nvalid == 16 && (reinterpret_cast<uintptr_t>(src) & 15) == 0) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float4 v = reinterpret_cast<const float4*>(src)[q];
      x[4 * q] = v.x;
      x[4 * q + 1] = v.y;
      x[4 * q + 2] = v.z;
      x[4 * q + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int j = 0; j < 16; ++j) x[j] = (j < nvalid) ? src[j * ks] : 0.0f;
  }
  uint32_t packed[NT][8];
#pragma unroll
  for (int j = 0; j < 16; j += 2) {
    uint32_t t0[NT], t1[NT];
    split_terms<NT>(x[j], t0);
    split_terms<NT>(x[j + 1], t1);
#pragma unroll
    for (int i = 0; i < NT; ++i) packed[i][j / 2] = t0[i] | (t1[i] << 16);
  }
  __nv_bfloat16* dst = planes + r * pitch + k0;
  if (nvalid == 16) {
#pragma unroll
    for (int i = 0; i < NT; ++i) {
      uint4* d4 = reinterpret_cast<uint4*>(dst + i * plane);
      d4[0] = make_uint4(packed[i][0], packed[i][1], packed[i][2], packed[i][3]);
      d4[1] = make_uint4(packed[i][4], packed[i][5], packed[i][6], packed[i][7]);
    }
  } else {   // unrolled with a predicate: the packed terms stay in registers
    unsigned short* d2 = reinterpret_cast<unsigned short*>(dst);
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      if (j < nvalid) {
#pragma unroll
        for (int i = 0; i < NT; ++i)
          d2[i * plane + j] = static_cast<unsigned short>(packed[i][j / 2] >> (16 * (j & 1)));
      }
    }
  }
}

// Rows contiguous (element (r, k) at X[r + k*ks]): a CTA converts a 64 x 64 tile through shared
// memory.  Warp w loads columns 8w..8w+7 (lanes along r: 128-byte loads); the terms go to
// [r][k] shared tiles; each warp then stores 8 rows x 128 B of every plane, and with DUAL also
// 8 k-rows x 128 B of the transposed planes [k][r] — whole lines in both layouts.
template <int NT, bool DUAL>
__global__ void __launch_bounds__(256) split_rc_tile_kernel(const float* __restrict__ X, int64_t R, int64_t Kd,
                                                            int64_t ks, __nv_bfloat16* __restrict__ planes,
                                                            int64_t pitch, __nv_bfloat16* __restrict__ planes_t,
                                                            int64_t pitch_t) {
  __shared__ float tile[64][65];                                 // [k][r]
  __shared__ __align__(16) unsigned short ts[NT][64][72];       // [term][r][k], 144-byte rows
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int64_t r0 = static_cast<int64_t>(blockIdx.x) * 64, k0 = static_cast<int64_t>(blockIdx.y) * 64;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int kk = w * 8 + c;
    const int64_t k = k0 + kk;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int rr = lane + 32 * h;
      const int64_t r = r0 + rr;
      tile[kk][rr] = (r < R && k < Kd) ? X[r + k * ks] : 0.0f;
    }
  }
  __syncthreads();
  const int rr = tid >> 2, kb = (tid & 3) * 16;   // this thread's row and 16-wide k chunk
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    uint32_t t[NT];
    split_terms<NT>(tile[kb + j][rr], t);
#pragma unroll
    for (int i = 0; i < NT; ++i) ts[i][rr][kb + j] = static_cast<unsigned short>(t[i]);
  }
  __syncthreads();
  {   // row-major planes [r][k]
    const int64_t r = r0 + rr, k = k0 + kb;
    if (r < R && k < Kd) {
      const int nvalid = static_cast<int>(Kd - k < 16 ? Kd - k : 16);
#pragma unroll
      for (int i = 0; i < NT; ++i) {
        unsigned short* d = reinterpret_cast<unsigned short*>(planes) + (i * R + r) * pitch + k;
        if (nvalid == 16) {
          const uint4* src = reinterpret_cast<const uint4*>(&ts[i][rr][kb]);
          reinterpret_cast<uint4*>(d)[0] = src[0];
          reinterpret_cast<uint4*>(d)[1] = src[1];
        } else {
          for (int j = 0; j < nvalid; ++j) d[j] = ts[i][rr][kb + j];
        }
      }
    }
  }
  if (DUAL) {   // transposed planes [k][r]: this thread's k row (tid >> 2) and 16-wide r chunk
    const int kk = tid >> 2, rb = (tid & 3) * 16;
    const int64_t k = k0 + kk, r = r0 + rb;
    if (k < Kd && r < R) {
      const int nvalid = static_cast<int>(R - r < 16 ? R - r : 16);
#pragma unroll
      for (int i = 0; i < NT; ++i) {
        unsigned short* d = reinterpret_cast<unsigned short*>(planes_t) + (i * Kd + k) * pitch_t + r;
        if (nvalid == 16) {
          uint32_t p[8];
#pragma unroll
          for (int q = 0; q < 8; ++q)
            p[q] = static_cast<uint32_t>(ts[i][rb + 2 * q][kk]) | (static_cast<uint32_t>(ts[i][rb + 2 * q + 1][kk]) << 16);
          reinterpret_cast<uint4*>(d)[0] = make_uint4(p[0], p[1], p[2], p[3]);
          reinterpret_cast<uint4*>(d)[1] = make_uint4(p[4], p[5], p[6], p[7]);
        } else {
          for (int q = 0; q < nvalid; ++q) d[q] = ts[i][rb + q][kk];
        }
      }
    }
  }
}

// BF16 term planes of the R x Kd operand whose element (r, k) is X[r*rs + k*ks]: planes
// [term][r][pitch] (and with planes_t, from the same read, [term][k][pitch_t]; rows contiguous
// only).  nterms = 2 or 3.
int split_bf16_terms(const float* X, int64_t R, int64_t Kd, int64_t rs, int64_t ks, int nterms,
                     __nv_bfloat16* planes, int64_t pitch, __nv_bfloat16* planes_t, int64_t pitch_t, int kind,
                     cudaStream_t s) {
  if (R <= 0 || Kd <= 0) return GB_OK;
  if (nterms != 2 && nterms != 3) return GB_ERR_INVALID_VALUE;
  if (rs == 1 || planes_t) {
    if (rs != 1) return GB_ERR_UNSUPPORTED;   // the transposed layout is written from row-contiguous X
    const int64_t ktiles = (Kd + 63) / 64;
    if (ktiles > 65535 || (R + 63) / 64 > 0x7FFFFFFF) return GB_ERR_UNSUPPORTED;
    dim3 grid(static_cast<unsigned>((R + 63) / 64), static_cast<unsigned>(ktiles));
    if (planes_t && nterms == 2)
      GB_LAUNCH(kind, s, (split_rc_tile_kernel<2, true><<<grid, 256, 0, s>>>(X, R, Kd, ks, planes, pitch, planes_t,
                                                                               pitch_t)));
    else if (planes_t)
      GB_LAUNCH(kind, s, (split_rc_tile_kernel<3, true><<<grid, 256, 0, s>>>(X, R, Kd, ks, planes, pitch, planes_t,
                                                                               pitch_t)));
    else if (nterms == 2)
      GB_LAUNCH(kind, s, (split_rc_tile_kernel<2, false><<<grid, 256, 0, s>>>(X, R, Kd, ks, planes, pitch, nullptr,
                                                                                0)));
    else
      GB_LAUNCH(kind, s, (split_rc_tile_kernel<3, false><<<grid, 256, 0, s>>>(X, R, Kd, ks, planes, pitch, nullptr,
                                                                                0)));
  } else {
    const int64_t kchunks = (Kd + 15) / 16;
    const int64_t plane = R * pitch;
    for (int64_t r0 = 0; r0 < R; r0 += 65535) {   // rows beyond the grid's y range: bands
      const int64_t rb = (R - r0 < 65535) ? R - r0 : 65535;
      dim3 grid(static_cast<unsigned>((kchunks + 255) / 256), static_cast<unsigned>(rb));
      if (nterms == 2)
        GB_LAUNCH(kind, s, (split_kc_kernel<2><<<grid, 256, 0, s>>>(X + r0 * rs, rb, Kd, rs, ks, planes + r0 * pitch,
                                                                    pitch, plane)));
      else
        GB_LAUNCH(kind, s, (split_kc_kernel<3><<<grid, 256, 0, s>>>(X + r0 * rs, rb, Kd, rs, ks, planes + r0 * pitch,
                                                                    pitch, plane)));
    }
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

static inline int64_t pitch64(int64_t k) { return ((k + 63) / 64) * 64; }
static inline size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

// Schedule of the 3xBF16 product: one group, pairs (hi,hi), (hi,lo), (lo,hi).
static void split3_schedule(SliceSchedule& S, int kb_chunk) {
  std::memset(&S, 0, sizeof(S));
  S.ngroups = 1;
  S.kb_chunk = kb_chunk;
  S.bits = 0;
  S.level[0] = 0;
  S.npairs[0] = 3;
  S.pair_off[0] = 0;
  S.pp[0] = 0; S.pq[0] = 0;
  S.pp[1] = 0; S.pq[1] = 1;
  S.pp[2] = 1; S.pq[2] = 0;
}

// Workspace layout for an adjoint of A (M x K), B (K x N), dC (M x N).
size_t adjoint_workspace_bytes(int64_t M, int64_t N, int64_t K) {
  const int64_t pN = pitch64(N), pM = pitch64(M);
  return al256(2 * static_cast<size_t>(M) * pN * 2) + al256(2 * static_cast<size_t>(K) * pN * 2) +
         al256(2 * static_cast<size_t>(K) * pM * 2) + al256(2 * static_cast<size_t>(N) * pM * 2);
}

int adjoint_f32(int64_t M, int64_t N, int64_t K, const float* A, int64_t lda, const float* B, int64_t ldb,
                const float* dC, int64_t lddc, float* dA, int64_t ldda, float* dB, int64_t lddb, void* ws,
                int sms, DeviceStatus* status, uint64_t wait_limit_ns, cudaStream_t s) {
  const int64_t pN = pitch64(N), pM = pitch64(M);
  char* w = static_cast<char*>(ws);
  __nv_bfloat16* P1 = reinterpret_cast<__nv_bfloat16*>(w);                      // dC [p][i][j]
  w += al256(2 * static_cast<size_t>(M) * pN * 2);
  __nv_bfloat16* P2 = reinterpret_cast<__nv_bfloat16*>(w);                      // B  [p][k][j]
  w += al256(2 * static_cast<size_t>(K) * pN * 2);
  __nv_bfloat16* P3 = reinterpret_cast<__nv_bfloat16*>(w);                      // A  [p][k][i]
  w += al256(2 * static_cast<size_t>(K) * pM * 2);
  __nv_bfloat16* P4 = reinterpret_cast<__nv_bfloat16*>(w);                      // dC [p][j][i]

  // dC (M x N, column-major): rows i contiguous -> [p][i][j] and, from the same read, [p][j][i]
  int rc = split_bf16_terms(dC, M, N, 1, lddc, 2, P1, pN, P4, pM, GB_KERNEL_ADJOINT_SPLIT, s);
  // B (K x N): rows k contiguous -> [p][k][j]
  if (!rc) rc = split_bf16_terms(B, K, N, 1, ldb, 2, P2, pN, nullptr, 0, GB_KERNEL_ADJOINT_SPLIT, s);
  // A^T rows k (contraction over i, contiguous in memory) -> [p][k][i]
  if (!rc) rc = split_bf16_terms(A, K, M, lda, 1, 2, P3, pM, nullptr, 0, GB_KERNEL_ADJOINT_SPLIT, s);
  if (rc) return rc;

  CUtensorMap ta0, tb0, ta1, tb1;
  rc = make_plane_tmap(&ta0, P1, N, M, 2, pN, TC_BM);
  if (!rc) rc = make_plane_tmap(&tb0, P2, N, K, 2, pN, TC_BN);
  if (!rc) rc = make_plane_tmap(&ta1, P3, M, K, 2, pM, TC_BM);
  if (!rc) rc = make_plane_tmap(&tb1, P4, M, N, 2, pM, TC_BN);
  if (rc) return rc;

  const int64_t big = M > N ? (M > K ? M : K) : (N > K ? N : K);
  const TcTuning tune = tc_tuning_for(TC_KIND_ADJOINT, big, big);
  const bool pair = tune.engine == 2;
  const int64_t tbm = pair ? 256 : TC_BM, tbn = pair ? 256 : TC_BN;
  TcParams prm;
  std::memset(&prm, 0, sizeof(prm));
  prm.band = tune.band;
  TcProblem& P = prm.prob[0];   // dA (M x K), contraction N
  P.M = M; P.N = K; P.K = N;
  P.tiles_m = static_cast<int32_t>((M + tbm - 1) / tbm);
  P.tiles_n = static_cast<int32_t>((K + tbn - 1) / tbn);
  P.tile_begin = 0;
  P.kb_total = static_cast<int32_t>((N + TC_BK - 1) / TC_BK);
  P.nchunks = 1;
  P.C = dA; P.ldc = ldda;
  P.alpha = 1.0; P.beta = 0.0;
  TcProblem& Q = prm.prob[1];   // dB (K x N), contraction M
  Q.M = K; Q.N = N; Q.K = M;
  Q.tiles_m = static_cast<int32_t>((K + tbm - 1) / tbm);
  Q.tiles_n = static_cast<int32_t>((N + tbn - 1) / tbn);
  Q.tile_begin = P.tiles_m * P.tiles_n;
  Q.kb_total = static_cast<int32_t>((M + TC_BK - 1) / TC_BK);
  Q.nchunks = 1;
  Q.C = dB; Q.ldc = lddb;
  Q.alpha = 1.0; Q.beta = 0.0;
  prm.nprob = 2;
  prm.total_tiles = Q.tile_begin + Q.tiles_m * Q.tiles_n;
  prm.tws = nullptr;
  prm.status = status;
  prm.wait_limit_ns = wait_limit_ns;
  SliceSchedule sched;
  split3_schedule(sched, P.kb_total > Q.kb_total ? P.kb_total : Q.kb_total);
  if (pair) {
    CUtensorMap tb0h, tb1h;   // 128-row B boxes: each CTA of a pair loads half of the B tile
    rc = make_plane_tmap(&tb0h, P2, N, K, 2, pN, 128);
    if (!rc) rc = make_plane_tmap(&tb1h, P4, M, N, 2, pM, 128);
    if (rc) return rc;
    CUtensorMap tc0, tc1;
    prm.c_tma = (tune.tma_store && make_c_tmap_f32(&tc0, dA, M, K, ldda) && make_c_tmap_f32(&tc1, dB, K, N, lddb))
                    ? 1 : 0;
    const int64_t ctas = 2 * static_cast<int64_t>(prm.total_tiles), cap = sms & ~1;
    return tc_gemm_pair_launch(TC_EPI_F32, ta0, tb0h, &ta1, &tb1h, sched, prm,
                               static_cast<int>(ctas < cap ? ctas : cap), GB_KERNEL_ADJOINT_MMA, s,
                               prm.c_tma ? &tc0 : nullptr, prm.c_tma ? &tc1 : nullptr);
  }
  const int grid = prm.total_tiles < sms ? prm.total_tiles : sms;
  return tc_gemm_launch(TC_EPI_F32, ta0, tb0, &ta1, &tb1, sched, prm, grid, GB_KERNEL_ADJOINT_MMA, s);
}

}  // namespace gb
