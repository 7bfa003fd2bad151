// Tuning table of the tensor-core engine: one launch configuration per kind of product and
// output-size class (the role jBLAS gives pick_kernel_size and BLASOptions,
// src/kernel_structure.jl:76-99 and src/blas_options.jl:2-7, but chosen by measurement:
// gb_autotune_tc times the candidates on the device, the host layer persists the winners).
#include <atomic>
#include <mutex>

#include "gb_common.cuh"
#include "tc_gemm.cuh"

namespace gb {

namespace {
std::mutex g_tune_mu;
bool g_tune_init = false;
TcTuning g_tune[TC_KINDS][TC_TUNE_CLASSES];

void init_locked() {
  if (g_tune_init) return;
  for (int k = 0; k < TC_KINDS; ++k)
    for (int c = 0; c < TC_TUNE_CLASSES; ++c) g_tune[k][c] = tc_default_tuning(k, c);
  g_tune_init = true;
}
}  // namespace

int tc_tune_class(int64_t M, int64_t N) {
  const int64_t d = M > N ? M : N;
  return d <= 2048 ? 0 : d <= 8192 ? 1 : 2;
}

// Defaults measured on GB300: CTA pairs (per-SM operand traffic halved, 95-100% of the BF16
// peak against 75% for one CTA per tile), bands of 8 pair tiles (2048 rows), direct stores;
// CRT products wider than 2048 columns in three column panels (narrow first and last panels
// where they add no round of the product kernel, else two equal ones: 0.993-0.994x the time of
// two equal panels at 8192^3, 0.986x at 12288^3, the same call at 4096^3 and 16384^3).
TcTuning tc_default_tuning(int kind, int cls) {
  TcTuning t;
  t.engine = 2;
  t.band = 8;
  t.tma_store = 0;
  t.panels = (kind == TC_KIND_CRT && cls > 0) ? 3 : 0;
  return t;
}

int tc_validate_tuning(int kind, const TcTuning& t) {
  if (kind < 0 || kind >= TC_KINDS) return GB_ERR_INVALID_VALUE;
  if (t.engine != 1 && t.engine != 2) return GB_ERR_INVALID_VALUE;
  if (kind == TC_KIND_CRT && t.engine != 2) return GB_ERR_INVALID_VALUE;   // CRT epilogue: pairs only
  if (t.band < 1 || t.band > 64) return GB_ERR_INVALID_VALUE;
  if (t.tma_store != 0 && t.tma_store != 1) return GB_ERR_INVALID_VALUE;
  if (t.tma_store && kind != TC_KIND_F32 && kind != TC_KIND_ADJOINT) return GB_ERR_INVALID_VALUE;
  if (t.tma_store && t.engine != 2) return GB_ERR_INVALID_VALUE;   // TMA-store epilogue: pair engine
  if (t.panels < 0 || t.panels > TC_MAX_PANELS || (t.panels > 1 && kind != TC_KIND_CRT)) return GB_ERR_INVALID_VALUE;
  return GB_OK;
}

TcTuning tc_tuning_for(int kind, int64_t M, int64_t N) {
  TcTuning t;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    init_locked();
    t = g_tune[kind][tc_tune_class(M, N)];
  }
  const int ov = tc_engine_setting();
  if (ov == 1 || ov == 2) {
    if (ov != t.engine && kind != TC_KIND_CRT) {
      // the band is counted in the engine's own tile rows: keep the rows per band
      t.band = ov == 1 ? t.band * 2 : (t.band + 1) / 2;
      if (t.band > 64) t.band = 64;
      t.engine = ov;
      if (ov == 1) t.tma_store = 0;
    }
  }
  return t;
}

int tc_set_tuning(int kind, int cls, const TcTuning* t) {
  if (kind < 0 || kind >= TC_KINDS || cls < 0 || cls >= TC_TUNE_CLASSES) return GB_ERR_INVALID_VALUE;
  const TcTuning v = t ? *t : tc_default_tuning(kind, cls);
  const int rc = tc_validate_tuning(kind, v);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  init_locked();
  g_tune[kind][cls] = v;
  return GB_OK;
}

TcTuning tc_get_tuning(int kind, int cls) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  init_locked();
  return g_tune[kind][cls];
}

}  // namespace gb

// ============================================================== autotuner
namespace gb {

// Seeded synthetic operands on the device: uniform [-1, 1) (dist 0) or sign * U[1,2) * 2^e with
// e uniform in [-8, 8] (dist 1, the emulated-FP64 inputs), from a splitmix64 hash of the index.
template <typename T>
__global__ void tune_fill_kernel(T* __restrict__ x, int64_t n, uint64_t seed, int dist) {
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    uint64_t z = seed + static_cast<uint64_t>(i) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    const double u = static_cast<double>(z >> 11) * 0x1p-53;   // [0, 1)
    double v;
    if (dist == 0) {
      v = 2.0 * u - 1.0;
    } else {
      const int e = static_cast<int>((z >> 3) % 17) - 8;
      v = ldexp(1.0 + u, e) * ((z & 1) ? -1.0 : 1.0);
    }
    x[i] = static_cast<T>(v);
  }
}

template <typename T>
static int tune_fill(T* x, int64_t n, uint64_t seed, int dist, cudaStream_t s) {
  if (n <= 0) return GB_OK;
  tune_fill_kernel<T><<<1024, 256, 0, s>>>(x, n, seed, dist);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

int tc_autotune(int kind, int64_t M, int64_t N, int64_t K, int reps, TcTuning* out, float* best_ms, cudaStream_t s) {
  if (kind < 0 || kind >= TC_KINDS || M < 1 || N < 1 || K < 1 || !out) return GB_ERR_INVALID_VALUE;
  if (reps < 1) reps = 1;
  const bool f64 = (kind == TC_KIND_SLICES || kind == TC_KIND_CRT);
  const size_t es = f64 ? 8 : 4;
  // operands: A (M x K), B (K x N), C (M x N); the adjoint also takes dB (K x N) as output
  const size_t na = static_cast<size_t>(M) * K, nb = static_cast<size_t>(K) * N, nc = static_cast<size_t>(M) * N;
  void *A = nullptr, *B = nullptr, *C = nullptr, *D = nullptr;
  GB_CUDA_TRY(cudaMallocAsync(&A, na * es, s));
  GB_CUDA_TRY(cudaMallocAsync(&B, nb * es, s));
  GB_CUDA_TRY(cudaMallocAsync(&C, nc * es, s));
  if (kind == TC_KIND_ADJOINT) GB_CUDA_TRY(cudaMallocAsync(&D, (na > nb ? na : nb) * es, s));
  int rc = f64 ? tune_fill(static_cast<double*>(A), static_cast<int64_t>(na), 1, 1, s)
               : tune_fill(static_cast<float*>(A), static_cast<int64_t>(na), 1, 0, s);
  if (!rc) rc = f64 ? tune_fill(static_cast<double*>(B), static_cast<int64_t>(nb), 2, 1, s)
                    : tune_fill(static_cast<float*>(B), static_cast<int64_t>(nb), 2, 0, s);
  if (!rc && kind == TC_KIND_ADJOINT) rc = tune_fill(static_cast<float*>(C), static_cast<int64_t>(nc), 3, 0, s);
  auto call = [&]() -> int {
    switch (kind) {
      case TC_KIND_SLICES:
        return gb_gemm_f64(0, 0, M, N, K, 1.0, static_cast<double*>(A), M, static_cast<double*>(B), K, 0.0,
                           static_cast<double*>(C), M, GB_MODE_OZAKI_BF16, 8, nullptr, s);
      case TC_KIND_CRT:
        return gb_gemm_f64(0, 0, M, N, K, 1.0, static_cast<double*>(A), M, static_cast<double*>(B), K, 0.0,
                           static_cast<double*>(C), M, GB_MODE_OZAKI_CRT, 15, nullptr, s);
      case TC_KIND_F32:
        return gb_gemm_f32_ex(0, 0, M, N, K, 1.0f, static_cast<float*>(A), M, static_cast<float*>(B), K, 0.0f,
                              static_cast<float*>(C), M, GB_MODE_BF16X3, s);
      default:   // adjoint of C = A B with dC = C: dA (M x K) into A's shape, dB (K x N) into D
        return gb_gemm_adjoint_f32(M, N, K, static_cast<float*>(A), M, static_cast<float*>(B), K,
                                   static_cast<float*>(C), M, static_cast<float*>(D), M, static_cast<float*>(D), K, s);
    }
  };
  // the adjoint writes dA over D as well as dB: both outputs share D's storage here, which only
  // the timing sees (the operands stay A, B, C)
  const int cls = tc_tune_class(M, N);
  const TcTuning saved = tc_get_tuning(kind, cls);
  const int saved_engine = tc_engine_setting();
  tc_set_engine(0);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (!rc && cudaEventCreate(&e0) != cudaSuccess) rc = GB_ERR_CUDA;
  if (!rc && cudaEventCreate(&e1) != cudaSuccess) rc = GB_ERR_CUDA;
  TcTuning best = saved;
  float best_t = 1e30f;
  for (int engine = 1; engine <= 2 && !rc; ++engine) {
    if (kind == TC_KIND_CRT && engine == 1) continue;
    for (int bi = 0; bi < 5 && !rc; ++bi) {
      const int band = (engine == 2 ? 2 : 4) << bi;   // 2..32 pair tiles, 4..64 single tiles
      // the second option: TMA stores of C (FP32 outputs on pairs) or column panels (CRT: 1..4)
      const int nopt = (kind == TC_KIND_CRT) ? TC_MAX_PANELS
                       : (engine == 2 && (kind == TC_KIND_F32 || kind == TC_KIND_ADJOINT)) ? 2 : 1;
      for (int opt = 0; opt < nopt && !rc; ++opt) {
        TcTuning t;
        t.engine = engine;
        t.band = band;
        t.tma_store = (kind == TC_KIND_CRT) ? 0 : opt;
        t.panels = (kind == TC_KIND_CRT) ? opt + 1 : 0;
        rc = tc_set_tuning(kind, cls, &t);
        if (!rc) rc = call();   // warm-up
        if (rc) break;
        cudaEventRecord(e0, s);
        for (int r = 0; r < reps && !rc; ++r) rc = call();
        cudaEventRecord(e1, s);
        if (rc) break;
        if (cudaEventSynchronize(e1) != cudaSuccess) {
          rc = GB_ERR_CUDA;
          break;
        }
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        ms /= reps;
        if (ms < best_t) {
          best_t = ms;
          best = t;
        }
      }
    }
  }
  tc_set_tuning(kind, cls, &saved);
  tc_set_engine(saved_engine);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFreeAsync(A, s);
  cudaFreeAsync(B, s);
  cudaFreeAsync(C, s);
  if (D) cudaFreeAsync(D, s);
  if (!rc) {
    const int crc = gb_check_status(s);   // a timed-out wait in any candidate voids the tuning
    if (crc) rc = crc;
  }
  if (rc) return rc;
  *out = best;
  if (best_ms) *best_ms = best_t;
  return GB_OK;
}

}  // namespace gb
