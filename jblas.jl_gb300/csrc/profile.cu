// Launch counters and per-kernel-kind CUDA-event timers (the library's tracing layer).
//
// Every kernel launch of the library goes through prof_before / prof_after.  Counting is
// always on (one relaxed atomic add); timing is on between gb_profile_start and
// gb_profile_stop, when an event pair is recorded on the launching stream around each
// launch and the elapsed times are summed per kernel kind at stop.
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#include <vector>

#include "gb_common.cuh"
#include "profile.cuh"

namespace gb {

static std::atomic<long long> g_launches[GB_KERNEL_KINDS];
static std::atomic<bool> g_profiling{false};
static std::mutex g_prof_mu;

struct PendingTiming {
  int kind;
  cudaEvent_t start, stop;
};
static std::vector<PendingTiming> g_pending;
static std::vector<cudaEvent_t> g_event_pool;
// Per-thread start event between prof_before and prof_after of one launch.
static thread_local cudaEvent_t t_start = nullptr;

static cudaEvent_t take_event() {
  if (!g_event_pool.empty()) {
    cudaEvent_t e = g_event_pool.back();
    g_event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  return e;
}

void prof_before(int kind, cudaStream_t s) {
  (void)kind;
  if (!g_profiling.load(std::memory_order_relaxed)) return;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  t_start = take_event();
  if (t_start) cudaEventRecord(t_start, s);
}

void prof_count(int kind) { g_launches[kind].fetch_add(1, std::memory_order_relaxed); }

void prof_after(int kind, cudaStream_t s) {
  g_launches[kind].fetch_add(1, std::memory_order_relaxed);
  if (!g_profiling.load(std::memory_order_relaxed) || !t_start) return;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  cudaEvent_t stop = take_event();
  if (!stop) return;
  cudaEventRecord(stop, s);
  g_pending.push_back({kind, t_start, stop});
  t_start = nullptr;
}

}  // namespace gb

using namespace gb;

extern "C" {

const char* gb_kernel_kind_name(int kind) {
  static const char* names[GB_KERNEL_KINDS] = {
      "ozaki_stats", "ozaki_split", "ozaki_slice_mma", "native_gemm", "scale_c",
      "grouped_gemm", "adjoint_split", "adjoint_mma", "ozaki_combine", "semiring_gemm",
      "f32_split", "f32_mma", "reserved12", "reserved13", "reserved14", "reserved15"};
  if (kind < 0 || kind >= GB_KERNEL_KINDS) return "unknown";
  return names[kind];
}

int gb_launch_counts(long long* counts, int n) {
  if (!counts || n < 0) return GB_ERR_INVALID_VALUE;
  for (int i = 0; i < n && i < GB_KERNEL_KINDS; ++i) counts[i] = g_launches[i].load();
  return GB_OK;
}

int gb_profile_start(void) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  for (auto& p : g_pending) {
    g_event_pool.push_back(p.start);
    g_event_pool.push_back(p.stop);
  }
  g_pending.clear();
  g_profiling.store(true);
  return GB_OK;
}

int gb_profile_stop(double* ms, long long* launches, int n) {
  g_profiling.store(false);
  std::lock_guard<std::mutex> lk(g_prof_mu);
  if (ms)
    for (int i = 0; i < n; ++i) ms[i] = 0.0;
  if (launches)
    for (int i = 0; i < n; ++i) launches[i] = 0;
  int rc = GB_OK;
  for (auto& p : g_pending) {
    float t = 0.f;
    cudaError_t e = cudaEventSynchronize(p.stop);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, p.start, p.stop);
    if (e != cudaSuccess) {
      rc = gb_set_cuda_error(e, "profile events");
    } else if (p.kind < n) {
      if (ms) ms[p.kind] += t;
      if (launches) launches[p.kind] += 1;
    }
    g_event_pool.push_back(p.start);
    g_event_pool.push_back(p.stop);
  }
  g_pending.clear();
  return rc;
}

}  // extern "C"
