// C-ABI entry points of libgbblas (declared in include/gbblas.h).
//
// Argument checking follows BLAS conventions (the reference has none: jmul! relies on
// static sizes and @inbounds, src/gemm.jl:244,312).  Device workspace for the Ozaki
// path is taken from the stream-ordered allocator (cudaMallocAsync / cudaFreeAsync on
// the caller's stream), so concurrent calls on different streams never share scratch.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <vector>

#include "gb_common.cuh"
#include "grouped.cuh"
#include "native_gemm.cuh"
#include "ozaki.cuh"
#include "semiring.cuh"
#include "tc_gemm.cuh"

namespace gb {
int measure_fma_peaks(int sms, double* fp64_tflops, double* fp32_tflops);
int tc_autotune(int kind, int64_t M, int64_t N, int64_t K, int reps, TcTuning* out, float* best_ms, cudaStream_t s);
size_t gemm_f32_tc_workspace_bytes(int64_t M, int64_t N, int64_t K, int nterms);
int gemm_f32_tc(int ta, int tb, int64_t M, int64_t N, int64_t K, float alpha, const float* A, int64_t lda,
                const float* B, int64_t ldb, float beta, float* C, int64_t ldc, int nterms, void* ws, int sms,
                DeviceStatus* status, uint64_t wait_limit_ns, cudaStream_t s);
size_t adjoint_workspace_bytes(int64_t M, int64_t N, int64_t K);
int adjoint_f32(int64_t M, int64_t N, int64_t K, const float* A, int64_t lda, const float* B, int64_t ldb,
                const float* dC, int64_t lddc, float* dA, int64_t ldda, float* dB, int64_t lddb, void* ws,
                int sms, DeviceStatus* status, uint64_t wait_limit_ns, cudaStream_t s);
}  // namespace gb

static thread_local char g_last_detail[256];
static thread_local gb_ozaki_plan_t g_last_plan;

int gb_set_cuda_error(cudaError_t e, const char* what) {
  std::snprintf(g_last_detail, sizeof(g_last_detail), "%s: %s", what, cudaGetErrorString(e));
  if (e == cudaErrorMemoryAllocation) return GB_ERR_ALLOC;
  return GB_ERR_CUDA;
}

namespace gb {

static std::atomic<uint64_t> g_wait_limit_ns{4000000000ull};
static std::atomic<uint64_t> g_ozaki_tol_bits{0};
static std::atomic<int> g_ozaki_min_chunks{1};

// A high-priority stream with the events that fork a call's work onto it and join it back:
// a CRT call runs its residue products there while its own stream splits the next column panel
// and reconstructs the previous one.  A second stream copies the finished blocks of C of a
// host-buffer call to the host.  One call holds a lane at a time.
struct Lane {
  // fork and join per block of C; the statistics' fork and join; the plan; one for errors;
  // one per block for its copy to the host and the copies' join
  static constexpr int STATS_FORK = 2 * TC_MAX_PANELS, STATS_JOIN = STATS_FORK + 1, PLAN = STATS_FORK + 2,
                       ERROR_JOIN = STATS_FORK + 3, COPY = STATS_FORK + 4, COPY_JOIN = COPY + TC_MAX_PANELS,
                       EVENTS = COPY_JOIN + 1;
  cudaStream_t stream = nullptr;
  cudaStream_t copy = nullptr;
  cudaEvent_t ev[EVENTS] = {};
};

// The host C of a host-buffer call (pinned memory): a CRT call in blocks copies each block of C
// there on its lane's copy stream once the block is reconstructed, beside the products and
// reconstruction of the later blocks, and sets `done`; otherwise the caller copies C after the
// call.
struct HostSink {
  double* C = nullptr;
  int64_t ldc = 0;
  bool done = false;
};

struct DeviceInfo {
  bool init = false;
  int status_code = GB_OK;
  int sms = 0;
  DeviceStatus* status = nullptr;  // device-side status word
  cudaMemPool_t pool = nullptr;    // workspace pool, memory kept across calls
  std::mutex lane_mu;
  std::vector<Lane*> free_lanes;   // created on demand, kept until exit
};
static std::mutex g_dev_mu;
// One entry per device ordinal; entries are never moved, so a DeviceInfo* stays valid while
// other threads set up further devices.
static std::vector<std::unique_ptr<DeviceInfo>> g_devs;

// A lane of the current device (created on first need), or nullptr when none can be made;
// the call gives it back with give_lane once its work is enqueued.
static Lane* take_lane(DeviceInfo* d) {
  {
    std::lock_guard<std::mutex> lk(d->lane_mu);
    if (!d->free_lanes.empty()) {
      Lane* l = d->free_lanes.back();
      d->free_lanes.pop_back();
      return l;
    }
  }
  std::unique_ptr<Lane> l(new Lane);
  int least = 0, greatest = 0;
  if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) return nullptr;
  if (cudaStreamCreateWithPriority(&l->stream, cudaStreamNonBlocking, greatest) != cudaSuccess) return nullptr;
  if (cudaStreamCreateWithFlags(&l->copy, cudaStreamNonBlocking) != cudaSuccess) {
    cudaStreamDestroy(l->stream);
    return nullptr;
  }
  for (int i = 0; i < Lane::EVENTS; ++i) {
    if (cudaEventCreateWithFlags(&l->ev[i], cudaEventDisableTiming) != cudaSuccess) {
      for (int j = 0; j < i; ++j) cudaEventDestroy(l->ev[j]);
      cudaStreamDestroy(l->copy);
      cudaStreamDestroy(l->stream);
      return nullptr;
    }
  }
  return l.release();
}

static void give_lane(DeviceInfo* d, Lane* l) {
  if (!l) return;
  std::lock_guard<std::mutex> lk(d->lane_mu);
  d->free_lanes.push_back(l);
}

// Per-device setup: architecture check, SM count, status word.
static int device_info(DeviceInfo** out) {
  int dev = 0;
  GB_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_dev_mu);
  if (static_cast<int>(g_devs.size()) <= dev) g_devs.resize(dev + 1);
  if (!g_devs[dev]) g_devs[dev].reset(new DeviceInfo);
  DeviceInfo& d = *g_devs[dev];
  if (!d.init) {
    d.init = true;
    int major = 0, minor = 0;
    GB_CUDA_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    GB_CUDA_TRY(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
    GB_CUDA_TRY(cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev));
    if (major != 10 || minor != 3) {
      std::snprintf(g_last_detail, sizeof(g_last_detail),
                    "device %d is sm_%d%d; libgbblas carries sm_103a code only", dev, major, minor);
      d.status_code = GB_ERR_NO_DEVICE;
    } else {
      cudaError_t e = cudaMalloc(&d.status, sizeof(DeviceStatus));
      if (e == cudaSuccess) e = cudaMemset(d.status, 0, sizeof(DeviceStatus));
      if (e == cudaSuccess) {
        // A library-owned stream-ordered pool that keeps its memory: the Ozaki workspace
        // (digit planes, GB-sized at large shapes) is reused call after call instead of
        // being unmapped at every synchronisation.
        cudaMemPoolProps props;
        std::memset(&props, 0, sizeof(props));
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        e = cudaMemPoolCreate(&d.pool, &props);
        if (e == cudaSuccess) {
          uint64_t keep = UINT64_MAX;
          e = cudaMemPoolSetAttribute(d.pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
      }
      if (e != cudaSuccess) d.status_code = gb_set_cuda_error(e, "device setup");
    }
  }
  if (d.status_code != GB_OK) return d.status_code;
  *out = &d;
  return GB_OK;
}

// Takes the device status word (code exchanged with 0) into `out`.
__global__ void status_take_kernel(DeviceStatus* __restrict__ st, DeviceStatus* __restrict__ out) {
  DeviceStatus r;
  r.code = atomicExch(&st->code, 0);
  r.where = r.code ? st->where : 0;
  r.block = r.code ? st->block : 0;
  r.pad = 0;
  *out = r;
}

// Device or managed memory only: a host pointer handed to a kernel would fault.
static bool is_device_ptr(const void* p) {
  if (p == nullptr) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

static int check_gemm_args(int ta, int tb, int64_t M, int64_t N, int64_t K, int64_t lda, int64_t ldb,
                           int64_t ldc, const void* A, const void* B, const void* C, bool need_ab) {
  if ((ta != 0 && ta != 1) || (tb != 0 && tb != 1)) return GB_ERR_INVALID_VALUE;
  if (M < 0 || N < 0 || K < 0) return GB_ERR_INVALID_VALUE;
  const int64_t a_rows = ta ? K : M, b_rows = tb ? N : K;
  if (lda < (a_rows > 1 ? a_rows : 1)) return GB_ERR_INVALID_VALUE;
  if (ldb < (b_rows > 1 ? b_rows : 1)) return GB_ERR_INVALID_VALUE;
  if (ldc < (M > 1 ? M : 1)) return GB_ERR_INVALID_VALUE;
  if (M == 0 || N == 0) return GB_OK;
  if (!is_device_ptr(C)) return GB_ERR_INVALID_VALUE;
  if (need_ab && K > 0 && (!is_device_ptr(A) || !is_device_ptr(B))) return GB_ERR_INVALID_VALUE;
  return GB_OK;
}

// ------------------------------------------------------------------ tensor maps
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

int make_plane_tmap(CUtensorMap* map, const void* base, int64_t K, int64_t rows, int64_t slices,
                    int64_t pitch, int box_rows, int64_t plane_rows) {
  if (plane_rows == 0) plane_rows = rows;
  if (plane_rows < rows) return GB_ERR_INVALID_VALUE;
  auto fn = encode_fn();
  if (!fn) {
    std::snprintf(g_last_detail, sizeof(g_last_detail), "cuTensorMapEncodeTiled unavailable");
    return GB_ERR_CUDA;
  }
  cuuint64_t dims[3] = {static_cast<cuuint64_t>(K), static_cast<cuuint64_t>(rows),
                        static_cast<cuuint64_t>(slices)};
  cuuint64_t strides[2] = {static_cast<cuuint64_t>(pitch * 2),
                           static_cast<cuuint64_t>(plane_rows * pitch * 2)};
  cuuint32_t box[3] = {64u, static_cast<cuuint32_t>(box_rows), 1u};
  cuuint32_t estr[3] = {1u, 1u, 1u};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box,
                  estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    std::snprintf(g_last_detail, sizeof(g_last_detail), "cuTensorMapEncodeTiled failed (%d)",
                  static_cast<int>(r));
    return GB_ERR_CUDA;
  }
  return GB_OK;
}

bool make_c_tmap_f32(CUtensorMap* map, const void* C, int64_t M, int64_t N, int64_t ldc) {
  auto fn = encode_fn();
  if (!fn || !C || M < 1 || N < 1 || (reinterpret_cast<uintptr_t>(C) & 15) || (ldc & 3)) return false;
  if (M > 0x7FFFFFFF || N > 0x7FFFFFFF || ldc * 4 >= (int64_t(1) << 40)) return false;
  cuuint64_t dims[2] = {static_cast<cuuint64_t>(M), static_cast<cuuint64_t>(N)};
  cuuint64_t strides[1] = {static_cast<cuuint64_t>(ldc * 4)};
  cuuint32_t box[2] = {32u, 32u};
  cuuint32_t estr[2] = {1u, 1u};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(C), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The last CRT call's plan lives on the device until someone asks for it.
struct PendingCrtPlan {
  bool pending = false;
  CrtPlanRecord* record = nullptr;   // the tagged read-back copy of the call's plan
  unsigned long long seq = 0;
  cudaEvent_t done = nullptr;
  int64_t M = 0, N = 0, kb_total = 0, k_chunk = 0;
};
static thread_local PendingCrtPlan g_pending_crt;

// ------------------------------------------------------------------ Ozaki driver
static double ozaki_tolerance() {
  uint64_t b = g_ozaki_tol_bits.load();
  if (b == 0) return std::ldexp(1.0, -50);
  double t;
  std::memcpy(&t, &b, sizeof(t));
  return t;
}

// Host copy of the split statistics of both operands.
struct HostStats {
  int64_t K = 0;
  std::vector<unsigned long long> amax_a, amax_b;
  std::vector<double> sabs_a, sabs_b, ssq_a, ssq_b;
};

static int exp_of(unsigned long long bits) {
  if (bits >= 0x7FF0000000000000ull) return INT32_MAX;
  if (bits == 0) return 0;
  double a;
  std::memcpy(&a, &bits, sizeof(a));
  return std::ilogb(a) + 1;
}

// A-priori normwise bound ||C - C_exact||_F / (||A||_F ||B||_F) for a plan (alpha = 1,
// beta = 0), from the split statistics (row/column exponents e, f; sums of |.|; norms):
//   truncation  both operands cut after s digits, plus the dropped products p + q > s + 1
//   recombination  FP64 sum of the exact group results, smallest level first: each drain
//               rounds once, so a term is charged once per later partial sum
//   final       the power-of-two rescale is exact, the alpha product rounds once
// Norm inequalities used: ||diag(x) Y diag(z)||_F <= ||x||_2 ||z||_2 max|Y| style bounds on
// the integer digit products (|S| <= npairs * kc * 2^(2b-2)).
// Norms of the split statistics, gathered once per call.  All exponent sums are taken
// relative to 2^(emax_a + emax_b) so that extreme magnitudes neither overflow nor vanish.
struct BoundStats {
  bool nonfinite = false;
  double na = 0, nb = 0, EA = 0, EB = 0, SA = 0, SB = 0;  // scaled by 2^-ref_a, 2^-ref_b
  double sa_max = 0, sb_max = 0;   // max over rows of sum_k |x| 2^-e (upper bounds, unscaled)
};

static BoundStats bound_stats(const HostStats& h) {
  BoundStats r;
  int ref_a = -1100, ref_b = -1100;
  for (auto bits : h.amax_a) {
    const int e = exp_of(bits);
    if (e == INT32_MAX) r.nonfinite = true; else if (bits && e > ref_a) ref_a = e;
  }
  for (auto bits : h.amax_b) {
    const int e = exp_of(bits);
    if (e == INT32_MAX) r.nonfinite = true; else if (bits && e > ref_b) ref_b = e;
  }
  if (r.nonfinite) return r;
  // The device sums are FP32 sums of truncated values |x| 2^-e (e: the row's exponent) over
  // K terms: sum |x| <= s1 (1 + 2^-23) / (1 - K 2^-24) + K 2^-126 (flushed tiny terms), and
  // sum x^2 >= s2 / (1 + K 2^-23) — one-sided bounds, as the error bound needs.
  const double Kd = static_cast<double>(h.K);
  const double gk = Kd * std::ldexp(1.0, -24);
  // (the host sum of the K-slice partials adds at most a few ulps of FP64: 2^-40 slack)
  const double up = (gk < 0.5 ? (1.0 + std::ldexp(1.0, -23)) / (1.0 - gk) : 4.0) * (1.0 + std::ldexp(1.0, -40));
  const double down = (1.0 - std::ldexp(1.0, -40)) / (1.0 + 2.0 * gk);
  const double tiny = Kd * std::ldexp(1.0, -126);
  double e2a = 0, e2b = 0, na2 = 0, nb2 = 0, sa2 = 0, sb2 = 0;
  for (size_t i = 0; i < h.amax_a.size(); ++i) {
    if (!h.amax_a[i]) continue;
    const int e = exp_of(h.amax_a[i]);
    e2a += std::ldexp(1.0, 2 * (e - ref_a));
    const double sa = std::ldexp(h.sabs_a[i] * up + tiny, e - ref_a);
    sa2 += sa * sa;
    r.sa_max = std::max(r.sa_max, h.sabs_a[i] * up + tiny);
    na2 += std::ldexp(h.ssq_a[i] * down, 2 * (e - ref_a));
  }
  for (size_t j = 0; j < h.amax_b.size(); ++j) {
    if (!h.amax_b[j]) continue;
    const int e = exp_of(h.amax_b[j]);
    e2b += std::ldexp(1.0, 2 * (e - ref_b));
    const double sb = std::ldexp(h.sabs_b[j] * up + tiny, e - ref_b);
    sb2 += sb * sb;
    r.sb_max = std::max(r.sb_max, h.sabs_b[j] * up + tiny);
    nb2 += std::ldexp(h.ssq_b[j] * down, 2 * (e - ref_b));
  }
  r.na = std::sqrt(na2); r.nb = std::sqrt(nb2);
  r.EA = std::sqrt(e2a); r.EB = std::sqrt(e2b);
  r.SA = std::sqrt(sa2); r.SB = std::sqrt(sb2);
  return r;
}

static inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Statistics of both operands: run on the device; when `host` is set, copied back and the
// K-slice sums rescaled to each row's exponent (Sum_s sum_s 2^(e_s - e)) into HostStats.
struct OperandStats {
  char* ws = nullptr;
  OzRowStats a{}, b{};
};

// With a lane (and no host copies), B's statistics run on the lane beside A's on `s`, and `s`
// waits for them before it returns.
static int run_stats(DeviceInfo* dev, const double* A, int64_t M, int64_t a_rs, int64_t a_ks, const double* B,
                     int64_t N, int64_t b_rs, int64_t b_ks, int64_t K, bool sums, bool host, OperandStats* os,
                     HostStats* h, cudaStream_t s, Lane* lane = nullptr) {
  const int Sa = oz_stats_kslices(M, K, a_ks, dev->sms), Sb = oz_stats_kslices(N, K, b_ks, dev->sms);
  const int64_t pa = Sa * M, pb = Sb * N;
  const size_t amax_bytes = align256((M + N) * sizeof(unsigned long long));
  const size_t part_bytes = align256((pa + pb) * sizeof(int32_t));
  GB_CUDA_TRY(cudaMallocFromPoolAsync(reinterpret_cast<void**>(&os->ws), amax_bytes + 3 * part_bytes, dev->pool, s));
  os->a.amax_bits = reinterpret_cast<unsigned long long*>(os->ws);
  os->b.amax_bits = os->a.amax_bits + M;
  os->a.part_e = reinterpret_cast<int32_t*>(os->ws + amax_bytes);
  os->b.part_e = os->a.part_e + pa;
  os->a.part_sa = reinterpret_cast<float*>(os->ws + amax_bytes + part_bytes);
  os->b.part_sa = os->a.part_sa + pa;
  os->a.part_sq = reinterpret_cast<float*>(os->ws + amax_bytes + 2 * part_bytes);
  os->b.part_sq = os->a.part_sq + pa;
  os->a.kslices = Sa;
  os->b.kslices = Sb;
  if (lane && !host) {
    cudaError_t e = cudaEventRecord(lane->ev[Lane::STATS_FORK], s);   // after the workspace allocation
    if (e == cudaSuccess) e = cudaStreamWaitEvent(lane->stream, lane->ev[Lane::STATS_FORK], 0);
    if (e != cudaSuccess) return gb_set_cuda_error(e, "ozaki statistics fork");
    int rc = oz_row_stats(A, M, K, a_rs, a_ks, os->a, sums, s);
    const int rcb = oz_row_stats(B, N, K, b_rs, b_ks, os->b, sums, lane->stream);
    e = cudaEventRecord(lane->ev[Lane::STATS_JOIN], lane->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, lane->ev[Lane::STATS_JOIN], 0);
    if (!rc) rc = rcb;
    if (!rc && e != cudaSuccess) rc = gb_set_cuda_error(e, "ozaki statistics join");
    return rc;
  }
  int rc = oz_row_stats(A, M, K, a_rs, a_ks, os->a, sums || host, s);
  if (!rc) rc = oz_row_stats(B, N, K, b_rs, b_ks, os->b, sums || host, s);
  if (rc || !host) return rc;
  std::vector<unsigned long long> amax(M + N);
  std::vector<int32_t> pe(pa + pb);
  std::vector<float> psa(pa + pb), psq(pa + pb);
  cudaMemcpyAsync(amax.data(), os->a.amax_bits, (M + N) * 8, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(pe.data(), os->a.part_e, (pa + pb) * 4, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(psa.data(), os->a.part_sa, (pa + pb) * 4, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(psq.data(), os->a.part_sq, (pa + pb) * 4, cudaMemcpyDeviceToHost, s);
  const cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return gb_set_cuda_error(e, "ozaki statistics");
  h->K = K;
  auto combine = [&](int64_t R, int S, int64_t off_amax, int64_t off_part, std::vector<unsigned long long>& am,
                     std::vector<double>& sabs, std::vector<double>& ssq) {
    am.assign(amax.begin() + off_amax, amax.begin() + off_amax + R);
    sabs.assign(R, 0.0);
    ssq.assign(R, 0.0);
    for (int64_t i = 0; i < R; ++i) {
      const int er = exp_of(am[i]);
      if (er == INT32_MAX || am[i] == 0) continue;
      for (int sl = 0; sl < S; ++sl) {
        const int64_t o = off_part + static_cast<int64_t>(sl) * R + i;
        if (pe[o] == INT32_MAX) continue;
        sabs[i] += std::ldexp(static_cast<double>(psa[o]), pe[o] - er);
        ssq[i] += std::ldexp(static_cast<double>(psq[o]), 2 * (pe[o] - er));
      }
    }
  };
  combine(M, Sa, 0, 0, h->amax_a, h->sabs_a, h->ssq_a);
  combine(N, Sb, M, pa, h->amax_b, h->sabs_b, h->ssq_b);
  return GB_OK;
}

static double ozaki_bound(const BoundStats& st, int64_t K, const OzPlan& plan) {
  if (st.nonfinite) return INFINITY;
  const double na = st.na, nb = st.nb;
  if (na == 0.0 || nb == 0.0) return 0.0;
  const double EA = st.EA, EB = st.EB, SA = st.SA, SB = st.SB;
  const int s = plan.slices, b = plan.bits;
  const double Kd = static_cast<double>(K);
  const double u = std::ldexp(1.0, -53);
  const double us = std::ldexp(1.0, -s * b);
  const double cs = (s - 1) / (1.0 - std::ldexp(1.0, -b));
  const double trunc = us * (EA * SB + EB * (SA + Kd * us * EA)) + Kd * us * cs * EA * EB;
  // leading (level-2) group: |digit_1 * w_1| <= |x| + 2^-b
  const double top = na * nb + std::ldexp(1.0, -b) * (EA * SB + EB * SA) + Kd * std::ldexp(1.0, -2 * b) * EA * EB;
  const int G = plan.sched.ngroups, nch = plan.nchunks;
  const double Kp = static_cast<double>(plan.k_chunk) * nch;
  const double D = static_cast<double>(G) * nch;
  double lower = 0.0;
  for (int g = 0; g < G; ++g) {
    const int level = plan.sched.level[g];
    if (level == 2) continue;
    const double coef = D - static_cast<double>(g) * nch;
    lower += coef * plan.sched.npairs[g] * Kp * std::ldexp(1.0, -(level - 2) * b);
  }
  const double recomb = u * (nch * top + lower * EA * EB);
  const double fin = u * top;
  return 1.01 * (trunc + recomb + fin) / (na * nb);
}

static int ozaki_gemm(DeviceInfo* dev, int ta, int tb, int64_t M, int64_t N, int64_t K, double alpha,
                      const double* A, int64_t lda, const double* B, int64_t ldb, double beta,
                      double* C, int64_t ldc, int slices, double* err_bound_out, cudaStream_t s) {
  if (slices < 0 || slices > OZ_MAX_SLICES) return GB_ERR_INVALID_VALUE;
  if ((M + TC_BM - 1) / TC_BM * ((N + TC_BN - 1) / TC_BN) > 0x7FFFFFFF) return GB_ERR_UNSUPPORTED;
  // op(A) rows i: X[i,k]; op(B) "rows" j: X[j,k] = op(B)[k,j]
  const int64_t a_rs = ta ? lda : 1, a_ks = ta ? 1 : lda;
  const int64_t b_rs = tb ? 1 : ldb, b_ks = tb ? ldb : 1;
  const int64_t pitch = ((K + 63) / 64) * 64;

  OperandStats os;
  HostStats h;
  const bool host_stats = (slices == 0 || err_bound_out);
  int rc = run_stats(dev, A, M, a_rs, a_ks, B, N, b_rs, b_ks, K, host_stats, host_stats, &os, &h, s);
  if (rc) {
    if (os.ws) cudaFreeAsync(os.ws, s);
    return rc;
  }
  char* st_ws = os.ws;
  OzRowStats& sa = os.a;
  OzRowStats& sb = os.b;

  OzPlan plan;
  int s_use = slices;
  if (host_stats) {
    const BoundStats bst = bound_stats(h);
    if (slices == 0) {
      // Cheapest plan (slices, K chunking -> digit width) whose bound meets the tolerance.
      const double tol = ozaki_tolerance();
      double best_cost = 0.0;
      bool found = false;
      for (int chunks = 1; chunks <= 8; chunks *= 2) {
        for (int cand = 1; cand <= OZ_MAX_SLICES; ++cand) {
          OzPlan p;
          if (oz_make_plan_chunks(M, N, K, cand, chunks, &p)) break;
          if (ozaki_bound(bst, K, p) > tol) continue;
          const double c = oz_plan_cost(p);
          if (!found || c < best_cost) {
            best_cost = c;
            plan = p;
            found = true;
          }
          break;   // more slices only cost more at this chunking
        }
      }
      if (!found) {   // tolerance out of reach: the most slices the split supports
        rc = GB_ERR_UNSUPPORTED;
        for (int cand = OZ_MAX_SLICES; cand >= 1 && rc; --cand) rc = oz_make_plan(M, N, K, cand, &plan);
      }
      s_use = plan.slices;
    } else {
      rc = oz_make_plan_chunks(M, N, K, s_use, g_ozaki_min_chunks.load(), &plan);
    }
    if (rc) {
      cudaFreeAsync(st_ws, s);
      return rc;
    }
    if (err_bound_out) *err_bound_out = ozaki_bound(bst, K, plan);
  } else {
    rc = oz_make_plan_chunks(M, N, K, s_use, g_ozaki_min_chunks.load(), &plan);
    if (rc) {
      cudaFreeAsync(st_ws, s);
      return rc;
    }
  }

  g_pending_crt.pending = false;
  g_last_plan.slices = plan.slices;
  g_last_plan.bits = plan.bits;
  g_last_plan.k_chunk = static_cast<int32_t>(plan.k_chunk);
  g_last_plan.products = plan.products;
  g_last_plan.groups = plan.groups;
  g_last_plan.flops_tensor = plan.flops_tensor;
  const TcTuning tune = tc_tuning_for(TC_KIND_SLICES, M, N);
  const int grid = oz_grid_for(dev->sms, M, N, tune.engine);
  const size_t pa_bytes = align256(static_cast<size_t>(s_use) * M * pitch * 2);
  const size_t pb_bytes = align256(static_cast<size_t>(s_use) * N * pitch * 2);
  const size_t ex_bytes = align256((M + N) * sizeof(int32_t));
  const size_t tw_bytes = (plan.groups * plan.nchunks > 1)
                              ? static_cast<size_t>(grid) * TC_BM * TC_BN * sizeof(double)
                              : 0;
  char* ws = nullptr;
  cudaError_t e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&ws), pa_bytes + pb_bytes + ex_bytes + tw_bytes,
                                          dev->pool, s);
  if (e != cudaSuccess) {
    cudaFreeAsync(st_ws, s);
    return gb_set_cuda_error(e, "ozaki workspace");
  }
  __nv_bfloat16* pa = reinterpret_cast<__nv_bfloat16*>(ws);
  __nv_bfloat16* pb = reinterpret_cast<__nv_bfloat16*>(ws + pa_bytes);
  int32_t* ea = reinterpret_cast<int32_t*>(ws + pa_bytes + pb_bytes);
  int32_t* eb = ea + M;
  double* tws = tw_bytes ? reinterpret_cast<double*>(ws + pa_bytes + pb_bytes + ex_bytes) : nullptr;

  rc = oz_split(A, M, K, a_rs, a_ks, sa.amax_bits, s_use, plan.bits, pa, pitch, ea, s);
  if (!rc) rc = oz_split(B, N, K, b_rs, b_ks, sb.amax_bits, s_use, plan.bits, pb, pitch, eb, s);
  if (!rc) {
    OzGemmArgs ga;
    ga.planes_a = pa;
    ga.planes_b = pb;
    ga.pitch = pitch;
    ga.slices = s_use;
    ga.M = M;
    ga.N = N;
    ga.K = K;
    ga.ea = ea;
    ga.eb = eb;
    ga.alpha = alpha;
    ga.beta = beta;
    ga.C = C;
    ga.ldc = ldc;
    ga.tws = tws;
    ga.status = dev->status;
    ga.wait_limit_ns = g_wait_limit_ns.load();
    ga.grid = grid;
    ga.engine = tune.engine;
    ga.band = tune.band;
    rc = oz_gemm_launch(ga, plan, s);
  }
  cudaFreeAsync(ws, s);
  cudaFreeAsync(st_ws, s);
  return rc;
}

// ------------------------------------------------------------------ CRT driver
// Column panels of a CRT call, in 256-column tiles: widths w[0..pcol) summing to tiles_n.
// The residue-product kernel runs one pair tile per CTA pair at a time, so a launch of t tiles
// takes ceil(t / pairs) rounds; panels may split C only where that adds no round over one launch.
// Three panels are a narrow first panel (the first products wait for a sliver of B's split),
// a wide middle one and a last one twice as wide as the first (its products run beside the
// middle panel's reconstruction, and a sliver of C is reconstructed after them): widths
// (e, tiles_n - 3e, 2e) for the smallest e that adds no round (8192 x 8192: 2, 26 and 4 tiles
// = 1 + 11 + 2 rounds, as one launch of 1024 tiles on 76 pairs); otherwise, and for other
// panel counts, equal panels, and two when three equal ones would add rounds.
// A host-buffer call copies each panel of C to the host once it is reconstructed, so there
// three panels are two halves and a narrow last panel, (w, w, e) for the smallest e that adds no
// round (8192 x 8192: 14, 14 and 4 tiles = 6 + 6 + 2 rounds): the first half's copy runs
// beside the second half's products, the second's beside the last panel's, and only the
// narrow last panel's copy follows the products.
// Returns the panel count used.
static int crt_panel_widths(int64_t tiles_m, int64_t tiles_n, int64_t pairs, int pcol, bool host_copies,
                            int64_t* w) {
  auto rounds = [&](int64_t cols) { return (tiles_m * cols + pairs - 1) / pairs; };
  const int64_t best = rounds(tiles_n);
  if (pcol == 3 && host_copies) {
    for (int64_t e = 1; 5 * e <= tiles_n; ++e) {
      const int64_t w0 = (tiles_n - e) / 2, w1 = tiles_n - e - w0;
      if (rounds(w0) + rounds(w1) + rounds(e) == best) {
        w[0] = w0;
        w[1] = w1;
        w[2] = e;
        return 3;
      }
    }
  }
  if (pcol == 3) {
    for (int64_t e = 1; 5 * e <= tiles_n; ++e) {
      if (rounds(e) + rounds(tiles_n - 3 * e) + rounds(2 * e) == best) {
        w[0] = e;
        w[1] = tiles_n - 3 * e;
        w[2] = 2 * e;
        return 3;
      }
    }
    int64_t eq = 0;
    for (int p = 0; p < 3; ++p) eq += rounds(tiles_n * (p + 1) / 3 - tiles_n * p / 3);
    if (eq > best) pcol = 2;
  }
  for (int p = 0; p < pcol; ++p) w[p] = tiles_n * (p + 1) / pcol - tiles_n * p / pcol;
  return pcol;
}

// The blocks of C a CRT call cuts an M x N output into, on whole 256 x 256 tiles: for the
// tuning's `panels` (clamped to 1..TC_MAX_PANELS and to one per 256 columns), `panels` column
// panels (crt_panel_widths), or 2 x 2 blocks for 4, so that the first products wait only for
// half of A's split as well (column panels when M <= 256).  Row boundaries m0[0..prow],
// column boundaries n0[0..pcol].
struct CrtBlocks {
  int prow = 1, pcol = 1;
  int64_t m0[3] = {}, n0[TC_MAX_PANELS + 1] = {};
};
static CrtBlocks crt_blocks(int64_t M, int64_t N, int panels, int sms, bool host_copies) {
  CrtBlocks b;
  const int64_t tiles_m = (M + 255) / 256, tiles_n = (N + 255) / 256;
  if (panels < 1) panels = 1;
  if (panels > TC_MAX_PANELS) panels = TC_MAX_PANELS;
  if (panels > tiles_n) panels = static_cast<int>(tiles_n > 0 ? tiles_n : 1);
  b.prow = (panels == 4 && tiles_m >= 2) ? 2 : 1;
  for (int p = 0; p <= b.prow; ++p) {
    const int64_t r = tiles_m * p / b.prow * 256;
    b.m0[p] = r < M ? r : M;
  }
  int64_t w[TC_MAX_PANELS];
  b.pcol = crt_panel_widths(tiles_m / b.prow, tiles_n, sms / 2 > 0 ? sms / 2 : 1, panels / b.prow, host_copies, w);
  for (int p = 0, t = 0; p < b.pcol; ++p) {
    t += static_cast<int>(w[p]);
    b.n0[p + 1] = static_cast<int64_t>(t) * 256 < N ? static_cast<int64_t>(t) * 256 : N;
  }
  return b;
}

// The plan (moduli n and integer bits t) is chosen on the device from the statistics
// (crt_plan_device), so an automatic call has no host round trip; the workspace is sized for
// the largest n the call may take.  The host only learns the plan when asked for it
// (err_bound_out, gb_last_ozaki_plan).

static int crt_gemm(DeviceInfo* dev, int ta, int tb, int64_t M, int64_t N, int64_t K, double alpha, const double* A,
                    int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc, int moduli,
                    double* err_bound_out, cudaStream_t s, HostSink* sink = nullptr) {
  if (moduli < 0 || moduli > TC_MAX_MODULI) return GB_ERR_INVALID_VALUE;
  if ((M + 255) / 256 * ((N + 255) / 256) > 0x7FFFFFFF) return GB_ERR_UNSUPPORTED;
  const int64_t a_rs = ta ? lda : 1, a_ks = ta ? 1 : lda;
  const int64_t b_rs = tb ? 1 : ldb, b_ks = tb ? ldb : 1;
  const int64_t pitch = ((K + 63) / 64) * 64;
  int t_fixed = 0;
  if (moduli > 0) {
    t_fixed = crt_bits_for(K, moduli);
    if (t_fixed < 1) return GB_ERR_UNSUPPORTED;   // too few moduli for this K
  }
  const int n_ws = moduli ? moduli : TC_MAX_MODULI;
  CrtPlan plan;   // K chunking and a schedule for up to n_ws moduli
  int rc = crt_make_plan(M, N, K, n_ws, t_fixed, &plan);
  if (rc) return rc;
  CrtPlanRecord* record = nullptr;
  unsigned long long seq = 0;
  rc = crt_plan_record(&record, &seq);
  if (rc) return rc;

  const bool sums = (moduli == 0 || err_bound_out);
  // Blocks of C: the residue products of block b run on a high-priority lane while this stream
  // splits the operand panels of block b + 1 and reconstructs block b - 1, on the SMs' spare
  // registers and issue slots beside the tensor-core kernel; before the first products, B's
  // statistics and first panel split run on the lane beside A's.  One block (the plain
  // sequence on this stream) when the tuning asks for one and under stream capture; at most
  // one block column per 256 columns.
  const TcTuning tune = tc_tuning_for(TC_KIND_CRT, M, N);
  const CrtBlocks blocks = crt_blocks(M, N, tune.panels, dev->sms, sink != nullptr);
  const int panels = blocks.prow * blocks.pcol;
  cudaStreamCaptureStatus cap_status = cudaStreamCaptureStatusNone;
  Lane* lane = nullptr;
  if (panels > 1 && cudaStreamIsCapturing(s, &cap_status) == cudaSuccess && cap_status == cudaStreamCaptureStatusNone)
    lane = take_lane(dev);
  struct LaneReturn {   // the lane goes back to the pool when the call has enqueued its work
    DeviceInfo* d;
    Lane* l;
    ~LaneReturn() { give_lane(d, l); }
  } lane_return{dev, lane};
  OperandStats os;
  HostStats h;
  rc = run_stats(dev, A, M, a_rs, a_ks, B, N, b_rs, b_ks, K, sums, false, &os, &h, s, lane);
  if (rc) {
    if (os.ws) cudaFreeAsync(os.ws, s);
    return rc;
  }
  CrtPlanParams pp;
  std::memset(&pp, 0, sizeof(pp));
  pp.M = M;
  pp.N = N;
  pp.K = K;
  pp.n_fixed = moduli;
  pp.t_fixed = t_fixed;
  pp.with_sums = sums ? 1 : 0;
  pp.tol = ozaki_tolerance();
  for (int n = 1; n <= TC_MAX_MODULI; ++n) {
    pp.log2m[n] = crt_log2_product(n);
    pp.tk[n] = crt_bits_for(K, n);
  }
  // The call's workspace: its plan record (read by its kernels only), residue planes of A and
  // B, residue-product planes and the row/column exponents.
  const int64_t mpad = (M + 255) / 256 * 256, npad = (N + 255) / 256 * 256;
  const size_t plan_bytes = align256(sizeof(CrtDevicePlan));
  const size_t pa_bytes = align256(static_cast<size_t>(n_ws) * M * pitch * 2);
  const size_t pb_bytes = align256(static_cast<size_t>(n_ws) * N * pitch * 2);
  const size_t res_bytes = align256(static_cast<size_t>(n_ws) * mpad * npad);
  const size_t ex_bytes = align256((M + N) * sizeof(int32_t));
  char* ws = nullptr;
  cudaError_t e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&ws),
                                          plan_bytes + pa_bytes + pb_bytes + res_bytes + ex_bytes, dev->pool, s);
  if (e != cudaSuccess) {
    cudaFreeAsync(os.ws, s);
    return gb_set_cuda_error(e, "ozaki crt workspace");
  }
  CrtDevicePlan* plan_d = reinterpret_cast<CrtDevicePlan*>(ws);
  char* wsp = ws + plan_bytes;
  void* scratch = nullptr;
  e = cudaMallocFromPoolAsync(&scratch, crt_plan_scratch_bytes(), dev->pool, s);
  if (e != cudaSuccess) {
    cudaFreeAsync(ws, s);
    cudaFreeAsync(os.ws, s);
    return gb_set_cuda_error(e, "ozaki crt planner scratch");
  }
  rc = crt_plan_device(os.a, os.b, pp, plan_d, record, seq, scratch, s);
  cudaFreeAsync(scratch, s);
  if (!rc && lane) {   // the lane's first split reads the plan
    const cudaError_t e = cudaEventRecord(lane->ev[Lane::PLAN], s);
    if (e != cudaSuccess) rc = gb_set_cuda_error(e, "ozaki crt plan event");
  }
  if (!rc && err_bound_out) {
    CrtDevicePlan hp;
    e = cudaMemcpyAsync(&hp, plan_d, sizeof(hp), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = gb_set_cuda_error(e, "ozaki crt plan");
    else *err_bound_out = hp.bound;
  }
  if (rc) {
    cudaFreeAsync(ws, s);
    cudaFreeAsync(os.ws, s);
    return rc;
  }
  __nv_bfloat16* pa = reinterpret_cast<__nv_bfloat16*>(wsp);
  __nv_bfloat16* pb = reinterpret_cast<__nv_bfloat16*>(wsp + pa_bytes);
  uint8_t* res = reinterpret_cast<uint8_t*>(wsp + pa_bytes + pb_bytes);
  int32_t* ea = reinterpret_cast<int32_t*>(wsp + pa_bytes + pb_bytes + res_bytes);
  int32_t* eb = ea + M;
  CrtGemmArgs ga;
  ga.planes_a = pa;
  ga.planes_b = pb;
  ga.pitch = pitch;
  ga.M = M;
  ga.N = N;
  ga.K = K;
  ga.ea = ea;
  ga.eb = eb;
  ga.alpha = alpha;
  ga.beta = beta;
  ga.C = C;
  ga.ldc = ldc;
  ga.res = res;
  ga.res_ld = mpad;
  ga.res_plane = mpad * npad;
  ga.status = dev->status;
  ga.wait_limit_ns = g_wait_limit_ns.load();
  ga.plan = plan_d;
  ga.band = tune.band;
  ga.a_plane_rows = M;
  ga.b_plane_rows = N;
  auto grid_for = [&](int64_t n) {
    const int64_t ctas = 2 * static_cast<int64_t>(tc_pair_tiles(M, n));
    const int64_t cap = dev->sms & ~1;
    return static_cast<int>(ctas < cap ? ctas : cap);
  };
  if (!lane) {
    rc = crt_split(A, M, K, a_rs, a_ks, os.a.amax_bits, plan_d, pa, pitch, M, ea, s);
    if (!rc) rc = crt_split(B, N, K, b_rs, b_ks, os.b.amax_bits, plan_d, pb, pitch, N, eb, s);
    if (!rc) {
      ga.grid = grid_for(N);
      rc = crt_mma_launch(ga, plan, s);
    }
    if (!rc) rc = crt_combine_launch(ga, s);
  } else {
    // Blocks of C (crt_blocks) run row by row; each split of a row panel of A or column panel
    // of B is enqueued on this stream just before the first block that needs it.
    const int prow = blocks.prow, pcol = blocks.pcol;
    const int64_t* m0 = blocks.m0;
    const int64_t* n0 = blocks.n0;
    auto block_args = [&](int r, int c) {
      CrtGemmArgs g = ga;
      g.M = m0[r + 1] - m0[r];
      g.N = n0[c + 1] - n0[c];
      g.planes_a = pa + m0[r] * pitch;
      g.a_plane_rows = M;
      g.planes_b = pb + n0[c] * pitch;
      g.ea = ea + m0[r];
      g.eb = eb + n0[c];
      g.C = C + m0[r] + n0[c] * ldc;
      g.res = res + m0[r] + n0[c] * mpad;
      const int64_t ctas = 2 * static_cast<int64_t>(tc_pair_tiles(g.M, g.N));
      const int64_t cap = dev->sms & ~1;
      g.grid = static_cast<int>(ctas < cap ? ctas : cap);
      return g;
    };
    cudaStream_t hs = lane->stream;
    auto cu = [&](cudaError_t e) {
      if (e != cudaSuccess && !rc) rc = gb_set_cuda_error(e, "ozaki crt panel pipeline");
    };
    bool a_done[2] = {false, false}, b_done[TC_MAX_PANELS] = {};
    const int nblocks = prow * pcol;
    for (int b = 0; b < nblocks && !rc; ++b) {
      const int r = b / pcol, c = b % pcol;
      if (!rc && !b_done[c]) {   // the first block's B panel on the lane, beside A's split here
        cudaStream_t bs = (b == 0) ? hs : s;
        if (b == 0) cu(cudaStreamWaitEvent(hs, lane->ev[Lane::PLAN], 0));
        if (!rc)
          rc = crt_split(B + n0[c] * b_rs, n0[c + 1] - n0[c], K, b_rs, b_ks, os.b.amax_bits + n0[c], plan_d,
                         pb + n0[c] * pitch, pitch, N, eb + n0[c], bs);
        b_done[c] = true;
      }
      if (!rc && !a_done[r]) {
        rc = crt_split(A + m0[r] * a_rs, m0[r + 1] - m0[r], K, a_rs, a_ks, os.a.amax_bits + m0[r], plan_d,
                       pa + m0[r] * pitch, pitch, M, ea + m0[r], s);
        a_done[r] = true;
      }
      if (!rc) cu(cudaEventRecord(lane->ev[2 * b], s));
      if (!rc) cu(cudaStreamWaitEvent(hs, lane->ev[2 * b], 0));
      if (!rc) rc = crt_mma_launch(block_args(r, c), plan, hs);
      if (!rc) cu(cudaEventRecord(lane->ev[2 * b + 1], hs));
    }
    int copies = 0;   // blocks of C on their way to the host C
    for (int b = 0; b < nblocks && !rc; ++b) {
      const int r = b / pcol, c = b % pcol;
      cu(cudaStreamWaitEvent(s, lane->ev[2 * b + 1], 0));
      if (!rc) rc = crt_combine_launch(block_args(r, c), s);
      if (!rc && sink) {
        cu(cudaEventRecord(lane->ev[Lane::COPY + b], s));
        cu(cudaStreamWaitEvent(lane->copy, lane->ev[Lane::COPY + b], 0));
        if (!rc) {
          const int64_t rows = m0[r + 1] - m0[r], cols = n0[c + 1] - n0[c];
          cu(cudaMemcpy2DAsync(sink->C + m0[r] + n0[c] * sink->ldc, sink->ldc * sizeof(double),
                               C + m0[r] + n0[c] * ldc, ldc * sizeof(double), rows * sizeof(double), cols,
                               cudaMemcpyDeviceToHost, lane->copy));
          if (!rc) ++copies;
        }
      }
    }
    if (copies) {   // the caller's stream waits for the copies (its workspace holds C)
      if (cudaEventRecord(lane->ev[Lane::COPY_JOIN], lane->copy) == cudaSuccess)
        cudaStreamWaitEvent(s, lane->ev[Lane::COPY_JOIN], 0);
      if (!rc) sink->done = (copies == nblocks);
    }
    if (rc) {
      // join whatever reached the lane before the error, so the workspace is freed after it
      if (cudaEventRecord(lane->ev[Lane::ERROR_JOIN], hs) == cudaSuccess)
        cudaStreamWaitEvent(s, lane->ev[Lane::ERROR_JOIN], 0);
    }
  }
  if (!rc) {
    PendingCrtPlan& pd = g_pending_crt;
    if (!pd.done && cudaEventCreateWithFlags(&pd.done, cudaEventDisableTiming) != cudaSuccess) pd.done = nullptr;
    pd.pending = pd.done && cudaEventRecord(pd.done, s) == cudaSuccess;
    pd.record = record;
    pd.seq = seq;
    pd.M = M;
    pd.N = N;
    pd.kb_total = plan.kb_total;
    pd.k_chunk = plan.k_chunk;
  }
  cudaFreeAsync(ws, s);
  cudaFreeAsync(os.ws, s);
  return rc;
}

// Fills g_last_plan from the device plan of the last CRT call of this thread, if any.
static int resolve_pending_crt_plan() {
  PendingCrtPlan& pd = g_pending_crt;
  if (!pd.pending) return GB_OK;
  pd.pending = false;
  GB_CUDA_TRY(cudaEventSynchronize(pd.done));
  CrtPlanRecord rec;
  GB_CUDA_TRY(cudaMemcpy(&rec, pd.record, sizeof(rec), cudaMemcpyDeviceToHost));
  if (rec.seq != pd.seq) {   // CRT_PLAN_RING later calls on this device reused the record
    std::snprintf(g_last_detail, sizeof(g_last_detail),
                  "the plan of this thread's last CRT call was overwritten by %d later calls", CRT_PLAN_RING);
    return GB_ERR_INVALID_VALUE;
  }
  const CrtDevicePlan& hp = rec.plan;
  g_last_plan.slices = hp.n;
  g_last_plan.bits = hp.t;
  g_last_plan.k_chunk = static_cast<int32_t>(pd.k_chunk);
  g_last_plan.products = hp.n;
  g_last_plan.groups = hp.n;
  g_last_plan.flops_tensor = 2.0 * static_cast<double>(pd.M) * static_cast<double>(pd.N) *
                             static_cast<double>(pd.kb_total * TC_BK) * hp.n;
  return GB_OK;
}

}  // namespace gb

using namespace gb;

// ====================================================================== C ABI
// Semiring GEMM entry points: argument checks as gb_gemm_*, then the typed launcher.
template <typename T, typename Fn>
static int semiring_entry(Fn fn, int sr, int ta, int tb, int64_t M, int64_t N, int64_t K, const T* A, int64_t lda,
                          const T* B, int64_t ldb, int accumulate, T* C, int64_t ldc, void* stream) {
  DeviceInfo* dev = nullptr;
  int rc = device_info(&dev);
  if (rc) return rc;
  if (sr < 0 || sr >= GB_SEMIRINGS || (accumulate != 0 && accumulate != 1)) return GB_ERR_INVALID_VALUE;
  rc = check_gemm_args(ta, tb, M, N, K, lda, ldb, ldc, A, B, C, true);
  if (rc || M == 0 || N == 0) return rc;
  return fn(sr, ta, tb, M, N, K, A, lda, B, ldb, accumulate, C, ldc, static_cast<cudaStream_t>(stream));
}

// kernel! / initkernel! entry points: argument checks, then the onto-D chain or jmul!'s chain.
template <typename T, typename Onto, typename Init>
static int kernel_entry(Onto onto, Init init_fn, T* D, const T* A, const T* X, int64_t Mk, int64_t Pk,
                        int64_t sAD, int64_t sX, int64_t N, int init, void* stream) {
  DeviceInfo* dev = nullptr;
  int rc = device_info(&dev);
  if (rc) return rc;
  if (Mk < 0 || Pk < 0 || N < 0 || (init != 0 && init != 1)) return GB_ERR_INVALID_VALUE;
  if (sAD < (Mk > 1 ? Mk : 1) || sX < (N > 1 ? N : 1)) return GB_ERR_INVALID_VALUE;
  if (Mk == 0 || Pk == 0) return GB_OK;
  if (!is_device_ptr(D) || (N > 0 && (!is_device_ptr(A) || !is_device_ptr(X)))) return GB_ERR_INVALID_VALUE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (init) return init_fn(0, 0, Mk, Pk, N, T(1), A, sAD, X, sX, T(0), D, sAD, dev->sms, s);
  return onto(Mk, Pk, N, A, sAD, X, sX, D, sAD, dev->sms, s);
}

// Host-buffer products: upload the stored operands (packed, leading dimension = rows), run the
// device call on them, download C, synchronise, read the status word.  With a pinned host C
// the device call gets it as a sink (HostSink), and a call that already copied C (block by
// block) leaves nothing to download.
template <typename T, typename DeviceCall>
static int gemm_host(DeviceCall call, int ta, int tb, int64_t M, int64_t N, int64_t K, T alpha, const T* A,
                     int64_t lda, const T* B, int64_t ldb, T beta, T* C, int64_t ldc, void* stream) {
  DeviceInfo* dev = nullptr;
  int rc = device_info(&dev);
  if (rc) return rc;
  if ((ta != 0 && ta != 1) || (tb != 0 && tb != 1) || M < 0 || N < 0 || K < 0) return GB_ERR_INVALID_VALUE;
  const int64_t ra = ta ? K : M, ca = ta ? M : K, rb = tb ? N : K, cb = tb ? K : N;
  if (lda < (ra > 1 ? ra : 1) || ldb < (rb > 1 ? rb : 1) || ldc < (M > 1 ? M : 1)) return GB_ERR_INVALID_VALUE;
  if (M == 0 || N == 0) return GB_OK;
  const bool need_ab = K > 0 && alpha != T(0);
  if (!C || (need_ab && (!A || !B))) return GB_ERR_INVALID_VALUE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t sz = sizeof(T);
  const size_t a_bytes = need_ab ? align256(static_cast<size_t>(ra) * ca * sz) : 0;
  const size_t b_bytes = need_ab ? align256(static_cast<size_t>(rb) * cb * sz) : 0;
  const size_t c_bytes = align256(static_cast<size_t>(M) * N * sz);
  char* ws = nullptr;
  cudaError_t e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&ws), a_bytes + b_bytes + c_bytes, dev->pool, s);
  if (e != cudaSuccess) return gb_set_cuda_error(e, "host-buffer workspace");
  T* dA = reinterpret_cast<T*>(ws);
  T* dB = reinterpret_cast<T*>(ws + a_bytes);
  T* dC = reinterpret_cast<T*>(ws + a_bytes + b_bytes);
  const int64_t la = ra > 1 ? ra : 1, lb = rb > 1 ? rb : 1, lc = M > 1 ? M : 1;
  if (need_ab) {
    e = cudaMemcpy2DAsync(dA, la * sz, A, lda * sz, ra * sz, ca, cudaMemcpyDefault, s);
    if (e == cudaSuccess) e = cudaMemcpy2DAsync(dB, lb * sz, B, ldb * sz, rb * sz, cb, cudaMemcpyDefault, s);
  }
  if (e == cudaSuccess && beta != T(0)) e = cudaMemcpy2DAsync(dC, lc * sz, C, ldc * sz, M * sz, N, cudaMemcpyDefault, s);
  if (e != cudaSuccess) {
    cudaFreeAsync(ws, s);
    return gb_set_cuda_error(e, "host-buffer upload");
  }
  HostSink sink;
  HostSink* sinkp = nullptr;
  cudaPointerAttributes attr;
  if (sizeof(T) == 8 && cudaPointerGetAttributes(&attr, C) == cudaSuccess && attr.type == cudaMemoryTypeHost) {
    sink.C = reinterpret_cast<double*>(C);
    sink.ldc = ldc;
    sinkp = &sink;
  }
  cudaGetLastError();   // an unregistered pointer is not an error here
  rc = call(ta, tb, M, N, K, alpha, need_ab ? dA : nullptr, la, need_ab ? dB : nullptr, lb, beta, dC, lc, stream,
            sinkp);
  if (!rc && !sink.done) {
    e = cudaMemcpy2DAsync(C, ldc * sz, dC, lc * sz, M * sz, N, cudaMemcpyDefault, s);
    if (e != cudaSuccess) rc = gb_set_cuda_error(e, "host-buffer download");
  }
  cudaFreeAsync(ws, s);
  e = cudaStreamSynchronize(s);
  if (!rc && e != cudaSuccess) rc = gb_set_cuda_error(e, "host-buffer call");
  if (!rc) rc = gb_check_status(stream);
  return rc;
}

extern "C" {

const char* gb_status_string(int status) {
  switch (status) {
    case GB_OK: return "ok";
    case GB_ERR_INVALID_VALUE: return "invalid value (size, leading dimension, flag or pointer)";
    case GB_ERR_UNSUPPORTED: return "unsupported on this device or build";
    case GB_ERR_PIPELINE_TIMEOUT: return "on-device pipeline wait timed out; kernel exited";
    case GB_ERR_CUDA: return g_last_detail[0] ? g_last_detail : "CUDA error";
    case GB_ERR_ALLOC: return "device workspace allocation failed";
    case GB_ERR_NO_DEVICE: return g_last_detail[0] ? g_last_detail : "no usable sm_103 device";
    default: return "unknown status";
  }
}

int gb_version(void) { return GBBLAS_VERSION; }

int gb_set_wait_limit_ns(uint64_t ns) {
  g_wait_limit_ns.store(ns == 0 ? 4000000000ull : ns);
  return GB_OK;
}

int gb_set_ozaki_tolerance(double tol) {
  if (!(tol >= 0.0)) return GB_ERR_INVALID_VALUE;
  uint64_t b = 0;
  if (tol > 0.0) std::memcpy(&b, &tol, sizeof(b));
  g_ozaki_tol_bits.store(b);
  return GB_OK;
}

static_assert(sizeof(gb_tc_tuning_t) == sizeof(TcTuning), "tuning layouts");

int gb_tc_size_class(int64_t M, int64_t N) {
  if (M < 0 || N < 0) return GB_ERR_INVALID_VALUE;
  return tc_tune_class(M, N);
}

int gb_tc_default_tuning(int kind, int size_class, gb_tc_tuning_t* out) {
  if (!out || kind < 0 || kind >= GB_TC_KINDS || size_class < 0 || size_class >= GB_TC_SIZE_CLASSES)
    return GB_ERR_INVALID_VALUE;
  const TcTuning t = tc_default_tuning(kind, size_class);
  std::memcpy(out, &t, sizeof(t));
  return GB_OK;
}

int gb_get_tc_tuning(int kind, int size_class, gb_tc_tuning_t* out) {
  if (!out || kind < 0 || kind >= GB_TC_KINDS || size_class < 0 || size_class >= GB_TC_SIZE_CLASSES)
    return GB_ERR_INVALID_VALUE;
  const TcTuning t = tc_get_tuning(kind, size_class);
  std::memcpy(out, &t, sizeof(t));
  return GB_OK;
}

int gb_set_tc_tuning(int kind, int size_class, const gb_tc_tuning_t* tuning) {
  if (!tuning) return tc_set_tuning(kind, size_class, nullptr);
  TcTuning t;
  std::memcpy(&t, tuning, sizeof(t));
  return tc_set_tuning(kind, size_class, &t);
}

int gb_autotune_tc(int kind, int64_t M, int64_t N, int64_t K, int reps, gb_tc_tuning_t* out, float* best_ms,
                   void* stream) {
  if (!out) return GB_ERR_INVALID_VALUE;
  DeviceInfo* dev = nullptr;
  int rc = device_info(&dev);
  if (rc) return rc;
  TcTuning t;
  rc = tc_autotune(kind, M, N, K, reps, &t, best_ms, static_cast<cudaStream_t>(stream));
  if (rc) return rc;
  std::memcpy(out, &t, sizeof(t));
  return GB_OK;
}

int gb_measure_fma_peaks(double* fp64_tflops, double* fp32_tflops) {
  DeviceInfo* dev = nullptr;
  int rc = device_info(&dev);
  if (rc) return rc;
  return measure_fma_peaks(dev->sms, fp64_tflops, fp32_tflops);
}

int gb_release_workspace(void) {
  DeviceInfo* dev = nullptr;
  int rc = device_info(&dev);
  if (rc) return rc;
  GB_CUDA_TRY(cudaDeviceSynchronize());
  GB_CUDA_TRY(cudaMemPoolTrimTo(dev->pool, 0));
  return GB_OK;
}

int gb_set_tc_engine(int engine) {
  if (engine < 0 || engine > 2) return GB_ERR_INVALID_VALUE;
  tc_set_engine(engine);
  return GB_OK;
}

int gb_set_ozaki_min_chunks(int min_chunks) {
  if (min_chunks < 0 || min_chunks > 64) return GB_ERR_INVALID_VALUE;
  g_ozaki_min_chunks.store(min_chunks == 0 ? 1 : min_chunks);
  return GB_OK;
}

int gb_check_status(void* stream) {
  DeviceInfo* dev = nullptr;
  int rc = device_info(&dev);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // Read and clear in one atomic step on the device, into a slot of this call's own: an error
  // recorded while the check runs is either taken by it or left for the next check, never lost.
  DeviceStatus* slot = nullptr;
  GB_CUDA_TRY(cudaMallocFromPoolAsync(reinterpret_cast<void**>(&slot), sizeof(DeviceStatus), dev->pool, s));
  status_take_kernel<<<1, 1, 0, s>>>(dev->status, slot);
  cudaError_t e = cudaGetLastError();
  DeviceStatus h;
  std::memset(&h, 0, sizeof(h));
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, slot, sizeof(h), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(slot, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return gb_set_cuda_error(e, "status check");
  if (h.code != 0) {
    std::snprintf(g_last_detail, sizeof(g_last_detail), "pipeline wait at site %d timed out in block %d",
                  h.where, h.block);
    return h.code;
  }
  return GB_OK;
}

// gb_gemm_f64, with the host C of a host-buffer call (or nullptr).
static int gemm_f64(int transA, int transB, int64_t M, int64_t N, int64_t K, double alpha, const double* A,
                    int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc, int mode,
                    int slices, double* err_bound_out, void* stream, HostSink* sink) {
  if (mode != GB_MODE_NATIVE && mode != GB_MODE_OZAKI_BF16 && mode != GB_MODE_OZAKI_INT8 &&
      mode != GB_MODE_OZAKI_CRT)
    return GB_ERR_INVALID_VALUE;
  DeviceInfo* dev = nullptr;
  int rc = device_info(&dev);
  if (rc) return rc;
  rc = check_gemm_args(transA, transB, M, N, K, lda, ldb, ldc, A, B, C, alpha != 0.0);
  if (rc) return rc;
  if (mode == GB_MODE_OZAKI_INT8) {
    std::snprintf(g_last_detail, sizeof(g_last_detail),
                  "tcgen05.mma kind::i8 is not available on sm_103a");
    return GB_ERR_UNSUPPORTED;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (M == 0 || N == 0) {
    if (err_bound_out) *err_bound_out = 0.0;
    return GB_OK;
  }
  if (mode == GB_MODE_NATIVE || alpha == 0.0 || K == 0) {
    if (err_bound_out) {
      const double ku = static_cast<double>(K) * std::ldexp(1.0, -53);
      *err_bound_out = (alpha == 0.0 || K == 0) ? 0.0 : ku / (1.0 - ku);
    }
    return native_gemm_f64(transA, transB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, dev->sms, s);
  }
  if (mode == GB_MODE_OZAKI_CRT)
    return crt_gemm(dev, transA, transB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, slices, err_bound_out, s,
                    sink);
  return ozaki_gemm(dev, transA, transB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, slices,
                    err_bound_out, s);
}

int gb_gemm_f64(int transA, int transB, int64_t M, int64_t N, int64_t K, double alpha, const double* A,
                int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc, int mode,
                int slices, double* err_bound_out, void* stream) {
  return gemm_f64(transA, transB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, mode, slices, err_bound_out, stream,
                  nullptr);
}

int gb_gemm_f32(int transA, int transB, int64_t M, int64_t N, int64_t K, float alpha, const float* A,
                int64_t lda, const float* B, int64_t ldb, float beta, float* C, int64_t ldc, void* stream) {
  DeviceInfo* dev = nullptr;
  int rc = device_info(&dev);
  if (rc) return rc;
  rc = check_gemm_args(transA, transB, M, N, K, lda, ldb, ldc, A, B, C, alpha != 0.0f);
  if (rc) return rc;
  return native_gemm_f32(transA, transB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, dev->sms,
                         static_cast<cudaStream_t>(stream));
}

int gb_gemm_f32_ex(int transA, int transB, int64_t M, int64_t N, int64_t K, float alpha, const float* A,
                   int64_t lda, const float* B, int64_t ldb, float beta, float* C, int64_t ldc, int mode,
                   void* stream) {
  if (mode != GB_MODE_NATIVE && mode != GB_MODE_BF16X3 && mode != GB_MODE_BF16X6) return GB_ERR_INVALID_VALUE;
  DeviceInfo* dev = nullptr;
  int rc = device_info(&dev);
  if (rc) return rc;
  rc = check_gemm_args(transA, transB, M, N, K, lda, ldb, ldc, A, B, C, alpha != 0.0f);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // no product to form (alpha = 0, K = 0): C = beta C exactly as the native mode does it
  if (mode == GB_MODE_NATIVE || M == 0 || N == 0 || K == 0 || alpha == 0.0f)
    return native_gemm_f32(transA, transB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, dev->sms, s);
  if (tc_pair_tiles(M, N) > 0x7FFFFFFF / 2 || tc_tiles(M, N) > 0x7FFFFFFF / 2) return GB_ERR_UNSUPPORTED;
  const int nterms = (mode == GB_MODE_BF16X3) ? 2 : 3;
  void* ws = nullptr;
  GB_CUDA_TRY(cudaMallocFromPoolAsync(&ws, gemm_f32_tc_workspace_bytes(M, N, K, nterms), dev->pool, s));
  rc = gemm_f32_tc(transA, transB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, nterms, ws, dev->sms, dev->status,
                   g_wait_limit_ns.load(), s);
  cudaFreeAsync(ws, s);
  return rc;
}

int gb_kernel_f64(double* pD, const double* pA, const double* pX, int64_t Mk, int64_t Pk, int64_t stride_AD,
                  int64_t stride_X, int64_t N, int init, void* stream) {
  return kernel_entry<double>(native_kernel_onto_f64, native_gemm_f64, pD, pA, pX, Mk, Pk, stride_AD, stride_X, N,
                              init, stream);
}

int gb_kernel_f32(float* pD, const float* pA, const float* pX, int64_t Mk, int64_t Pk, int64_t stride_AD,
                  int64_t stride_X, int64_t N, int init, void* stream) {
  return kernel_entry<float>(native_kernel_onto_f32, native_gemm_f32, pD, pA, pX, Mk, Pk, stride_AD, stride_X, N,
                             init, stream);
}

int gb_gemm_adjoint_f32(int64_t M, int64_t N, int64_t K, const float* A, int64_t lda, const float* B,
                        int64_t ldb, const float* dC, int64_t lddc, float* dA, int64_t ldda, float* dB,
                        int64_t lddb, void* stream) {
  DeviceInfo* dev = nullptr;
  int rc = device_info(&dev);
  if (rc) return rc;
  if (M < 0 || N < 0 || K < 0) return GB_ERR_INVALID_VALUE;
  auto ld_ok = [](int64_t ld, int64_t rows) { return ld >= (rows > 1 ? rows : 1); };
  if (!ld_ok(lda, M) || !ld_ok(ldb, K) || !ld_ok(lddc, M) || !ld_ok(ldda, M) || !ld_ok(lddb, K))
    return GB_ERR_INVALID_VALUE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const bool need_da = M > 0 && K > 0, need_db = K > 0 && N > 0;
  if ((need_da && !is_device_ptr(dA)) || (need_db && !is_device_ptr(dB))) return GB_ERR_INVALID_VALUE;
  if (M == 0 || N == 0 || K == 0) {
    // an empty contraction gives zero gradients
    if (need_da) GB_CUDA_TRY(cudaMemset2DAsync(dA, ldda * sizeof(float), 0, M * sizeof(float), K, s));
    if (need_db) GB_CUDA_TRY(cudaMemset2DAsync(dB, lddb * sizeof(float), 0, K * sizeof(float), N, s));
    return GB_OK;
  }
  if (!is_device_ptr(A) || !is_device_ptr(B) || !is_device_ptr(dC)) return GB_ERR_INVALID_VALUE;
  if (static_cast<int64_t>(tc_tiles(M, K)) + tc_tiles(K, N) > 0x7FFFFFFF) return GB_ERR_UNSUPPORTED;
  void* ws = nullptr;
  GB_CUDA_TRY(cudaMallocFromPoolAsync(&ws, adjoint_workspace_bytes(M, N, K), dev->pool, s));
  rc = adjoint_f32(M, N, K, A, lda, B, ldb, dC, lddc, dA, ldda, dB, lddb, ws, dev->sms, dev->status,
                   g_wait_limit_ns.load(), s);
  cudaFreeAsync(ws, s);
  return rc;
}

int gb_grouped_default_tuning(int dtype_bytes, gb_grouped_tuning_t* out) {
  if (!out || (dtype_bytes != 4 && dtype_bytes != 8)) return GB_ERR_INVALID_VALUE;
  *out = grouped_default_tuning(dtype_bytes);
  return GB_OK;
}

size_t gb_grouped_workspace_size(int count) { return count < 0 ? 0 : grouped_workspace_bytes(count); }

static int grouped_call(int dtype_bytes, const gb_problem_t* problems, int count, const gb_grouped_tuning_t* tuning,
                        void* workspace, size_t workspace_bytes, void* stream) {
  DeviceInfo* dev = nullptr;
  int rc = device_info(&dev);
  if (rc) return rc;
  if (count < 0) return GB_ERR_INVALID_VALUE;
  if (count == 0) return GB_OK;
  if (!is_device_ptr(problems)) return GB_ERR_INVALID_VALUE;
  const gb_grouped_tuning_t t = tuning ? *tuning : grouped_default_tuning(dtype_bytes);
  rc = grouped_validate_tuning(dtype_bytes, t);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t need = grouped_workspace_bytes(count);
  void* ws = workspace;
  if (ws) {
    if (workspace_bytes < need || !is_device_ptr(ws) || (reinterpret_cast<uintptr_t>(ws) & 7))
      return GB_ERR_INVALID_VALUE;
  } else {
    GB_CUDA_TRY(cudaMallocFromPoolAsync(&ws, need, dev->pool, s));
  }
  rc = grouped_launch(dtype_bytes, problems, count, t, static_cast<long long*>(ws), dev->sms, s);
  if (!workspace) cudaFreeAsync(ws, s);
  return rc;
}

int gb_gemm_grouped_f64(const gb_problem_t* problems, int count, const gb_grouped_tuning_t* tuning,
                        void* workspace, size_t workspace_bytes, void* stream) {
  return grouped_call(8, problems, count, tuning, workspace, workspace_bytes, stream);
}

int gb_gemm_grouped_f32(const gb_problem_t* problems, int count, const gb_grouped_tuning_t* tuning,
                        void* workspace, size_t workspace_bytes, void* stream) {
  return grouped_call(4, problems, count, tuning, workspace, workspace_bytes, stream);
}

int gb_gemm_grouped_f64_noalloc(const gb_problem_t* problems, int count, const gb_grouped_tuning_t* tuning,
                                void* stream) {
  // A null or host table would fault in the prologue: reject it before any launch.
  if (count > 0 && count <= GB_GROUPED_NOALLOC_MAX && !is_device_ptr(problems)) return GB_ERR_INVALID_VALUE;
  return grouped_f64_noalloc(problems, count, tuning, static_cast<cudaStream_t>(stream));
}

static int strided_batched(int dtype_bytes, int64_t M, int64_t N, int64_t K, double alpha, const void* A,
                           int64_t lda, int64_t sa, const void* B, int64_t ldb, int64_t sb, double beta, void* C,
                           int64_t ldc, int64_t sc, int64_t count, void* stream) {
  DeviceInfo* dev = nullptr;
  int rc = device_info(&dev);
  if (rc) return rc;
  if (M < 0 || N < 0 || K < 0 || count < 0 || count > 0x7FFFFFFF || sa < 0 || sb < 0 || sc < 0)
    return GB_ERR_INVALID_VALUE;
  if (lda < (M > 1 ? M : 1) || ldb < (K > 1 ? K : 1) || ldc < (M > 1 ? M : 1)) return GB_ERR_INVALID_VALUE;
  if (count == 0 || M == 0 || N == 0) return GB_OK;
  if (count > 1 && sc < ldc * (N - 1) + M) return GB_ERR_INVALID_VALUE;   // C_i would overlap
  if (!is_device_ptr(C)) return GB_ERR_INVALID_VALUE;
  if (alpha != 0.0 && K > 0 && (!is_device_ptr(A) || !is_device_ptr(B))) return GB_ERR_INVALID_VALUE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int n = static_cast<int>(count);
  const size_t tab_bytes = (sizeof(gb_problem_t) * static_cast<size_t>(n) + 255) & ~size_t(255);
  const size_t ws_bytes = grouped_workspace_bytes(n);
  char* ws = nullptr;
  GB_CUDA_TRY(cudaMallocFromPoolAsync(reinterpret_cast<void**>(&ws), tab_bytes + ws_bytes, dev->pool, s));
  gb_problem_t* tab = reinterpret_cast<gb_problem_t*>(ws);
  rc = grouped_fill_strided(tab, n, M, N, K, lda, ldb, ldc, A, B, C, sa * dtype_bytes, sb * dtype_bytes,
                            sc * dtype_bytes, alpha, beta, s);
  if (!rc)
    rc = grouped_launch(dtype_bytes, tab, n, grouped_default_tuning(dtype_bytes),
                        reinterpret_cast<long long*>(ws + tab_bytes), dev->sms, s);
  cudaFreeAsync(ws, s);
  return rc;
}

int gb_gemm_strided_batched_f64(int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t lda,
                                int64_t strideA, const double* B, int64_t ldb, int64_t strideB, double beta,
                                double* C, int64_t ldc, int64_t strideC, int64_t count, void* stream) {
  return strided_batched(8, M, N, K, alpha, A, lda, strideA, B, ldb, strideB, beta, C, ldc, strideC, count, stream);
}

int gb_gemm_strided_batched_f32(int64_t M, int64_t N, int64_t K, float alpha, const float* A, int64_t lda,
                                int64_t strideA, const float* B, int64_t ldb, int64_t strideB, float beta,
                                float* C, int64_t ldc, int64_t strideC, int64_t count, void* stream) {
  return strided_batched(4, M, N, K, alpha, A, lda, strideA, B, ldb, strideB, beta, C, ldc, strideC, count, stream);
}

int gb_gemm_semiring_f64(int semiring, int transA, int transB, int64_t M, int64_t N, int64_t K, const double* A,
                         int64_t lda, const double* B, int64_t ldb, int accumulate, double* C, int64_t ldc,
                         void* stream) {
  return semiring_entry(semiring_gemm_f64, semiring, transA, transB, M, N, K, A, lda, B, ldb, accumulate, C, ldc,
                        stream);
}

int gb_gemm_semiring_f32(int semiring, int transA, int transB, int64_t M, int64_t N, int64_t K, const float* A,
                         int64_t lda, const float* B, int64_t ldb, int accumulate, float* C, int64_t ldc,
                         void* stream) {
  return semiring_entry(semiring_gemm_f32, semiring, transA, transB, M, N, K, A, lda, B, ldb, accumulate, C, ldc,
                        stream);
}

int gb_gemm_semiring_i32(int semiring, int transA, int transB, int64_t M, int64_t N, int64_t K, const int32_t* A,
                         int64_t lda, const int32_t* B, int64_t ldb, int accumulate, int32_t* C, int64_t ldc,
                         void* stream) {
  return semiring_entry(semiring_gemm_i32, semiring, transA, transB, M, N, K, A, lda, B, ldb, accumulate, C, ldc,
                        stream);
}

int gb_autotune_grouped(int dtype_bytes, const gb_problem_t* host_problems, int count, int reps,
                        gb_grouped_tuning_t* out, float* class_ms, void* stream) {
  if (!out || count < 0 || (count > 0 && !host_problems) || (dtype_bytes != 4 && dtype_bytes != 8))
    return GB_ERR_INVALID_VALUE;
  DeviceInfo* dev = nullptr;
  int rc = device_info(&dev);
  if (rc) return rc;
  return grouped_autotune(dtype_bytes, host_problems, count, dev->sms, dev->pool, reps < 1 ? 1 : reps, out,
                          class_ms, static_cast<cudaStream_t>(stream));
}

int gb_jmul_f64(double* D, const double* A, const double* X, int64_t M, int64_t N, int64_t P, void* stream) {
  return gb_gemm_f64(0, 0, M, P, N, 1.0, A, M > 1 ? M : 1, X, N > 1 ? N : 1, 0.0, D, M > 1 ? M : 1,
                     GB_MODE_NATIVE, 0, nullptr, stream);
}

int gb_jmul_f32(float* D, const float* A, const float* X, int64_t M, int64_t N, int64_t P, void* stream) {
  return gb_gemm_f32(0, 0, M, P, N, 1.0f, A, M > 1 ? M : 1, X, N > 1 ? N : 1, 0.0f, D, M > 1 ? M : 1,
                     stream);
}

int gb_gemm_f64_host(int transA, int transB, int64_t M, int64_t N, int64_t K, double alpha, const double* A,
                     int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc, int mode,
                     int slices, double* err_bound_out, void* stream) {
  auto call = [&](int ta, int tb, int64_t m, int64_t n, int64_t k, double al, const double* a, int64_t la,
                  const double* b, int64_t lb, double be, double* c, int64_t lc, void* st, HostSink* sink) {
    return gemm_f64(ta, tb, m, n, k, al, a, la, b, lb, be, c, lc, mode, slices, err_bound_out, st, sink);
  };
  return gemm_host<double>(call, transA, transB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, stream);
}

int gb_gemm_f32_host(int transA, int transB, int64_t M, int64_t N, int64_t K, float alpha, const float* A,
                     int64_t lda, const float* B, int64_t ldb, float beta, float* C, int64_t ldc, void* stream) {
  auto call = [&](int ta, int tb, int64_t m, int64_t n, int64_t k, float al, const float* a, int64_t la,
                  const float* b, int64_t lb, float be, float* c, int64_t lc, void* st, HostSink*) {
    return gb_gemm_f32(ta, tb, m, n, k, al, a, la, b, lb, be, c, lc, st);
  };
  return gemm_host<float>(call, transA, transB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, stream);
}

int gb_jmul_f64_host(double* D, const double* A, const double* X, int64_t M, int64_t N, int64_t P, void* stream) {
  return gb_gemm_f64_host(0, 0, M, P, N, 1.0, A, M > 1 ? M : 1, X, N > 1 ? N : 1, 0.0, D, M > 1 ? M : 1,
                          GB_MODE_NATIVE, 0, nullptr, stream);
}

int gb_jmul_f32_host(float* D, const float* A, const float* X, int64_t M, int64_t N, int64_t P, void* stream) {
  return gb_gemm_f32_host(0, 0, M, P, N, 1.0f, A, M > 1 ? M : 1, X, N > 1 ? N : 1, 0.0f, D, M > 1 ? M : 1,
                          stream);
}

int gb_last_ozaki_plan(gb_ozaki_plan_t* out) {
  if (!out) return GB_ERR_INVALID_VALUE;
  const int rc = resolve_pending_crt_plan();
  if (rc) return rc;
  *out = g_last_plan;
  return GB_OK;
}

int gb_plan_ozaki(int64_t M, int64_t N, int64_t K, int slices, gb_ozaki_plan_t* out) {
  if (!out || M < 0 || N < 0 || K < 0) return GB_ERR_INVALID_VALUE;
  OzPlan p;
  int rc = oz_make_plan(M, N, K, slices, &p);
  if (rc) return rc;
  out->slices = p.slices;
  out->bits = p.bits;
  out->k_chunk = static_cast<int32_t>(p.k_chunk);
  out->products = p.products;
  out->groups = p.groups;
  out->flops_tensor = p.flops_tensor;
  return GB_OK;
}

int gb_plan_ozaki_crt(int64_t M, int64_t N, int64_t K, int moduli, gb_ozaki_plan_t* out) {
  if (!out || M < 0 || N < 0 || K < 0 || moduli < 1 || moduli > TC_MAX_MODULI) return GB_ERR_INVALID_VALUE;
  CrtPlan p;
  const int rc = crt_make_plan(M, N, K, moduli, 0, &p);
  if (rc) return rc;
  out->slices = p.n;
  out->bits = p.t;
  out->k_chunk = static_cast<int32_t>(p.k_chunk);
  out->products = p.n;
  out->groups = p.n;
  out->flops_tensor = p.flops_tensor;
  return GB_OK;
}

int gb_crt_blocks(int64_t M, int64_t N, int panels, int sms, int host_copies, int64_t* rows, int* row_blocks,
                  int64_t* cols, int* col_blocks) {
  if (M < 1 || N < 1 || sms < 1 || (host_copies != 0 && host_copies != 1) || !rows || !row_blocks || !cols ||
      !col_blocks)
    return GB_ERR_INVALID_VALUE;
  if ((M + 255) / 256 > 0x7FFFFFFF / ((N + 255) / 256)) return GB_ERR_UNSUPPORTED;
  const CrtBlocks b = crt_blocks(M, N, panels, sms, host_copies != 0);
  *row_blocks = b.prow;
  *col_blocks = b.pcol;
  for (int p = 0; p <= b.prow; ++p) rows[p] = b.m0[p];
  for (int p = 0; p <= b.pcol; ++p) cols[p] = b.n0[p];
  return GB_OK;
}

}  // extern "C"
