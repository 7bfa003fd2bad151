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

__device__ __forceinline__ void split_hi_lo(float x, uint32_t& hi_bits, uint32_t& lo_bits) {
  const __nv_bfloat16 hi = __float2bfloat16_rn(x);
  const float r = x - __bfloat162float(hi);
  const __nv_bfloat16 lo = __float2bfloat16_rn(r);
  hi_bits = static_cast<uint32_t>(__bfloat16_as_ushort(hi));
  lo_bits = static_cast<uint32_t>(__bfloat16_as_ushort(lo));
}

// k contiguous or strided (element (r, k) at X[r*rs + k*ks]): one thread = one row r and 16
// consecutive k, neighbouring threads neighbouring k; writes planes[0] (hi) and planes[1] (lo),
// [plane][r][pitch], 32 bytes per plane per thread.  With ks == 1 the 16 values are read as four
// 16-byte loads when aligned.
__global__ void __launch_bounds__(256) split3_kc_kernel(const float* __restrict__ X, int64_t R, int64_t Kd,
                                                        int64_t rs, int64_t ks, __nv_bfloat16* __restrict__ planes,
                                                        int64_t pitch) {
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
  uint32_t hp[8], lp[8];
#pragma unroll
  for (int j = 0; j < 16; j += 2) {
    uint32_t h0, l0, h1, l1;
    split_hi_lo(x[j], h0, l0);
    split_hi_lo(x[j + 1], h1, l1);
    hp[j / 2] = h0 | (h1 << 16);
    lp[j / 2] = l0 | (l1 << 16);
  }
  const int64_t plane = R * pitch;
  __nv_bfloat16* dst = planes + r * pitch + k0;
  if (nvalid == 16) {
    uint4* h4 = reinterpret_cast<uint4*>(dst);
    uint4* l4 = reinterpret_cast<uint4*>(dst + plane);
    h4[0] = make_uint4(hp[0], hp[1], hp[2], hp[3]);
    h4[1] = make_uint4(hp[4], hp[5], hp[6], hp[7]);
    l4[0] = make_uint4(lp[0], lp[1], lp[2], lp[3]);
    l4[1] = make_uint4(lp[4], lp[5], lp[6], lp[7]);
  } else {   // unrolled with a predicate: hp / lp stay in registers
    unsigned short* d2 = reinterpret_cast<unsigned short*>(dst);
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      if (j < nvalid) {
        d2[j] = static_cast<unsigned short>(hp[j / 2] >> (16 * (j & 1)));
        d2[plane + j] = static_cast<unsigned short>(lp[j / 2] >> (16 * (j & 1)));
      }
    }
  }
}

// Rows contiguous (element (r, k) at X[r + k*ks]): a CTA converts a 64 x 64 tile through shared
// memory.  Warp w loads columns 8w..8w+7 (lanes along r: 128-byte loads); the hi/lo values go to
// [r][k] shared tiles; each warp then stores 8 rows x 128 B of both planes, and with DUAL also
// 8 k-rows x 128 B of the transposed planes [k][r] — whole lines in both layouts.
template <bool DUAL>
__global__ void __launch_bounds__(256) split3_rc_tile_kernel(const float* __restrict__ X, int64_t R, int64_t Kd,
                                                             int64_t ks, __nv_bfloat16* __restrict__ planes,
                                                             int64_t pitch, __nv_bfloat16* __restrict__ planes_t,
                                                             int64_t pitch_t) {
  __shared__ float tile[64][65];                              // [k][r]
  __shared__ __align__(16) unsigned short hs[64][72], ls[64][72];   // [r][k], 144-byte rows
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
    uint32_t hb, lb;
    split_hi_lo(tile[kb + j][rr], hb, lb);
    hs[rr][kb + j] = static_cast<unsigned short>(hb);
    ls[rr][kb + j] = static_cast<unsigned short>(lb);
  }
  __syncthreads();
  {   // row-major planes [r][k]
    const int64_t r = r0 + rr, k = k0 + kb;
    if (r < R && k < Kd) {
      const int nvalid = static_cast<int>(Kd - k < 16 ? Kd - k : 16);
      unsigned short* dh = reinterpret_cast<unsigned short*>(planes) + r * pitch + k;
      unsigned short* dl = dh + R * pitch;
      if (nvalid == 16) {
        const uint4* sh = reinterpret_cast<const uint4*>(&hs[rr][kb]);
        const uint4* sl = reinterpret_cast<const uint4*>(&ls[rr][kb]);
        reinterpret_cast<uint4*>(dh)[0] = sh[0];
        reinterpret_cast<uint4*>(dh)[1] = sh[1];
        reinterpret_cast<uint4*>(dl)[0] = sl[0];
        reinterpret_cast<uint4*>(dl)[1] = sl[1];
      } else {
        for (int j = 0; j < nvalid; ++j) {
          dh[j] = hs[rr][kb + j];
          dl[j] = ls[rr][kb + j];
        }
      }
    }
  }
  if (DUAL) {   // transposed planes [k][r]: this thread's k row (tid >> 2) and 16-wide r chunk
    const int kk = tid >> 2, rb = (tid & 3) * 16;
    const int64_t k = k0 + kk, r = r0 + rb;
    if (k < Kd && r < R) {
      const int nvalid = static_cast<int>(R - r < 16 ? R - r : 16);
      unsigned short* th = reinterpret_cast<unsigned short*>(planes_t) + k * pitch_t + r;
      unsigned short* tl = th + Kd * pitch_t;
      if (nvalid == 16) {
        uint32_t ph[8], pl[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          ph[i] = static_cast<uint32_t>(hs[rb + 2 * i][kk]) | (static_cast<uint32_t>(hs[rb + 2 * i + 1][kk]) << 16);
          pl[i] = static_cast<uint32_t>(ls[rb + 2 * i][kk]) | (static_cast<uint32_t>(ls[rb + 2 * i + 1][kk]) << 16);
        }
        reinterpret_cast<uint4*>(th)[0] = make_uint4(ph[0], ph[1], ph[2], ph[3]);
        reinterpret_cast<uint4*>(th)[1] = make_uint4(ph[4], ph[5], ph[6], ph[7]);
        reinterpret_cast<uint4*>(tl)[0] = make_uint4(pl[0], pl[1], pl[2], pl[3]);
        reinterpret_cast<uint4*>(tl)[1] = make_uint4(pl[4], pl[5], pl[6], pl[7]);
      } else {
        for (int i = 0; i < nvalid; ++i) {
          th[i] = hs[rb + i][kk];
          tl[i] = ls[rb + i][kk];
        }
      }
    }
  }
}

static int split3(const float* X, int64_t R, int64_t Kd, int64_t rs, int64_t ks, __nv_bfloat16* planes,
                  int64_t pitch, __nv_bfloat16* planes_t, int64_t pitch_t, cudaStream_t s) {
  if (R <= 0 || Kd <= 0) return GB_OK;
  const int64_t kchunks = (Kd + 15) / 16;
  if (rs == 1 || planes_t) {
    if (rs != 1) return GB_ERR_UNSUPPORTED;   // the transposed layout is written from row-contiguous X
    const int64_t ktiles = (Kd + 63) / 64;
    if (ktiles > 65535) return GB_ERR_UNSUPPORTED;
    dim3 grid(static_cast<unsigned>((R + 63) / 64), static_cast<unsigned>(ktiles));
    if (planes_t)
      GB_LAUNCH(GB_KERNEL_ADJOINT_SPLIT, s,
                (split3_rc_tile_kernel<true><<<grid, 256, 0, s>>>(X, R, Kd, ks, planes, pitch, planes_t, pitch_t)));
    else
      GB_LAUNCH(GB_KERNEL_ADJOINT_SPLIT, s,
                (split3_rc_tile_kernel<false><<<grid, 256, 0, s>>>(X, R, Kd, ks, planes, pitch, nullptr, 0)));
  } else {
    if (R > 65535) return GB_ERR_UNSUPPORTED;
    dim3 grid(static_cast<unsigned>((kchunks + 255) / 256), static_cast<unsigned>(R));
    GB_LAUNCH(GB_KERNEL_ADJOINT_SPLIT, s,
              (split3_kc_kernel<<<grid, 256, 0, s>>>(X, R, Kd, rs, ks, planes, pitch)));
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
  int rc = split3(dC, M, N, 1, lddc, P1, pN, P4, pM, s);
  // B (K x N): rows k contiguous -> [p][k][j]
  if (!rc) rc = split3(B, K, N, 1, ldb, P2, pN, nullptr, 0, s);
  // A^T rows k (contraction over i, contiguous in memory) -> [p][k][i]
  if (!rc) rc = split3(A, K, M, lda, 1, P3, pM, nullptr, 0, s);
  if (rc) return rc;

  CUtensorMap ta0, tb0, ta1, tb1;
  rc = make_plane_tmap(&ta0, P1, N, M, 2, pN, TC_BM);
  if (!rc) rc = make_plane_tmap(&tb0, P2, N, K, 2, pN, TC_BN);
  if (!rc) rc = make_plane_tmap(&ta1, P3, M, K, 2, pM, TC_BM);
  if (!rc) rc = make_plane_tmap(&tb1, P4, M, N, 2, pM, TC_BN);
  if (rc) return rc;

  const bool pair = tc_use_pair();
  const int64_t tbm = pair ? 256 : TC_BM, tbn = pair ? 256 : TC_BN;
  TcParams prm;
  std::memset(&prm, 0, sizeof(prm));
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
    const int64_t ctas = 2 * static_cast<int64_t>(prm.total_tiles), cap = sms & ~1;
    return tc_gemm_pair_launch(TC_EPI_F32, ta0, tb0h, &ta1, &tb1h, sched, prm,
                               static_cast<int>(ctas < cap ? ctas : cap), GB_KERNEL_ADJOINT_MMA, s);
  }
  const int grid = prm.total_tiles < sms ? prm.total_tiles : sms;
  return tc_gemm_launch(TC_EPI_F32, ta0, tb0, &ta1, &tb1, sched, prm, grid, GB_KERNEL_ADJOINT_MMA, s);
}

}  // namespace gb
