/*
 * CPU oracle for the blocked GEMM hot path of jBLAS.jl — TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline arm may load
 * this library, and only as the checker / the timed CPU reference.  The GPU
 * product path never calls into it.
 *
 * Parity status: UNPINNED by the reference's own tests.  jBLAS.jl ships no
 * golden vectors (test/runtests.jl has no assertions and no seeds) and the
 * package cannot run here (no Julia; src/cpu_info.jl is missing and
 * src/gemm.jl:260 reads an undefined global).  The arithmetic below is pinned
 * instead by (i) an independent pure-Python exact-rational restatement of the
 * same fma chain (tests/golden/make_golden.py), bit-exact, and (ii) two near-exact
 * dot products: a compensated one (Dot2) and one accumulated in IEEE binary128.
 *
 * Reference arithmetic restated here (paths relative to the jBLAS.jl tree):
 *   src/gemm.jl:71-91    initialize_block: D_rc = A[:,1] * X[1,c]   (a rounded product)
 *   src/gemm.jl:149-170  fma_increment_block: D_rc = fma(A[:,n], X[n,c], D_rc), n = 2..N
 *   src/gemm.jl:3-11     store_block: column-major store, leading dimension M
 *   src/gemm.jl:313-336  tile loop order (cc outer, rc inner); K runs in order 1..N
 * so every output element is  d = a_1*x_1;  d = fma(a_k, x_k, d) for k = 2..K,
 * one rounding per step, sequential K.  The loop order over tiles does not
 * change any element's value.
 *
 * Extensions beyond jmul! (the reference has only D = A*X):
 *   - remainder tiles are computed (jmul! skips them, src/gemm.jl:266-267,340-345);
 *   - alpha/beta:  C = alpha*acc           when beta == 0 (C is not read),
 *                  C = fma(alpha, acc, beta*C0) otherwise;
 *                  alpha == 0 gives C = beta*C0 (A, B not read), K == 0 gives acc = 0;
 *   - transposes via strides (op(A) = A or A^T, op(B) = B or B^T).
 *
 * Build: compiled with -ffp-contract=off so that only the explicit fma() calls fuse.
 */
#define _POSIX_C_SOURCE 199309L   /* clock_gettime */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef int64_t i64;

#define AIDX(tr, i, k, ld) ((tr) ? ((k) + (i) * (ld)) : ((i) + (k) * (ld)))
#define BIDX(tr, k, j, ld) ((tr) ? ((j) + (k) * (ld)) : ((k) + (j) * (ld)))

/* ---------------------------------------------------------------- naive fma chain */

/* The reference fma chain for one element (src/gemm.jl:76-89, 154-168). */
static inline double chain_f64(int ta, int tb, i64 i, i64 j, i64 K, const double* A, i64 lda,
                               const double* B, i64 ldb) {
  if (K == 0) return 0.0;
  double d = A[AIDX(ta, i, 0, lda)] * B[BIDX(tb, 0, j, ldb)];
  for (i64 k = 1; k < K; ++k) d = fma(A[AIDX(ta, i, k, lda)], B[BIDX(tb, k, j, ldb)], d);
  return d;
}
static inline float chain_f32(int ta, int tb, i64 i, i64 j, i64 K, const float* A, i64 lda,
                              const float* B, i64 ldb) {
  if (K == 0) return 0.0f;
  float d = A[AIDX(ta, i, 0, lda)] * B[BIDX(tb, 0, j, ldb)];
  for (i64 k = 1; k < K; ++k) d = fmaf(A[AIDX(ta, i, k, lda)], B[BIDX(tb, k, j, ldb)], d);
  return d;
}

/* C = alpha*op(A)*op(B) + beta*C, column-major, element order as jmul!. */
void or_gemm_f64(int ta, int tb, i64 M, i64 N, i64 K, double alpha, const double* A, i64 lda,
                 const double* B, i64 ldb, double beta, double* C, i64 ldc, int nthreads) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
#endif
  for (i64 j = 0; j < N; ++j)
    for (i64 i = 0; i < M; ++i) {
      double* c = &C[i + j * ldc];
      if (alpha == 0.0) { *c = (beta == 0.0) ? 0.0 : beta * *c; continue; }
      double acc = chain_f64(ta, tb, i, j, K, A, lda, B, ldb);
      *c = (beta == 0.0) ? alpha * acc : fma(alpha, acc, beta * *c);
    }
  (void)nthreads;
}

void or_gemm_f32(int ta, int tb, i64 M, i64 N, i64 K, float alpha, const float* A, i64 lda,
                 const float* B, i64 ldb, float beta, float* C, i64 ldc, int nthreads) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
#endif
  for (i64 j = 0; j < N; ++j)
    for (i64 i = 0; i < M; ++i) {
      float* c = &C[i + j * ldc];
      if (alpha == 0.0f) { *c = (beta == 0.0f) ? 0.0f : beta * *c; continue; }
      float acc = chain_f32(ta, tb, i, j, K, A, lda, B, ldb);
      *c = (beta == 0.0f) ? alpha * acc : fmaf(alpha, acc, beta * *c);
    }
  (void)nthreads;
}

/* jmul!(D, A, X): D (M x P) = A (M x N) * X (N x P); the reference's N is the contraction
 * dimension (src/gemm.jl:244).  Leading dimensions are M, N, M as for an MMatrix. */
void or_jmul_f64(double* D, const double* A, const double* X, i64 M, i64 N, i64 P) {
  or_gemm_f64(0, 0, M, P, N, 1.0, A, M, X, N, 0.0, D, M, 1);
}
void or_jmul_f32(float* D, const float* A, const float* X, i64 M, i64 N, i64 P) {
  or_gemm_f32(0, 0, M, P, N, 1.0f, A, M, X, N, 0.0f, D, M, 1);
}

/* kernel!(pD, pA, pX, Kernel{Mk,Pk,stride_AD,stride_X,N}) (src/kernels.jl:212-238): D (Mk x Pk,
 * leading dimension sAD) += A (Mk x N, sAD) * X (N x Pk, sX), per element
 * d = fma(a_n, x_n, d) for n = 1..N starting from D's value (the vmuladd chain).  init:
 * initkernel! (src/kernels.jl:240-273), d = a_1 * x_1 (rounded) first, D not read; N = 0
 * leaves D (init: 0). */
#define OR_KERNEL(NAME, T, FMA)                                                                     \
  void NAME(T* D, const T* A, const T* X, i64 Mk, i64 Pk, i64 sAD, i64 sX, i64 N, int init) {      \
    for (i64 p = 0; p < Pk; ++p)                                                                    \
      for (i64 m = 0; m < Mk; ++m) {                                                                \
        T d;                                                                                        \
        i64 n0 = 0;                                                                                 \
        if (init) {                                                                                 \
          if (N == 0) { D[m + p * sAD] = (T)0; continue; }                                          \
          d = A[m] * X[p * sX];                                                                     \
          n0 = 1;                                                                                   \
        } else {                                                                                    \
          d = D[m + p * sAD];                                                                       \
        }                                                                                           \
        for (i64 n = n0; n < N; ++n) d = FMA(A[m + n * sAD], X[n + p * sX], d);                     \
        D[m + p * sAD] = d;                                                                         \
      }                                                                                             \
  }
OR_KERNEL(or_kernel_f64, double, fma)
OR_KERNEL(or_kernel_f32, float, fmaf)

/* ------------------------------------------------- register-tiled timed baseline */
/*
 * The jmul! algorithm as the reference generates it: a TR x TC register tile whose shape
 * pick_kernel_size chooses for the host's register file (src/kernel_structure.jl:76-99,
 * restated by or_pick_kernel_size below and by oracle.pick_kernel_size), the full K
 * reduction held in the tile (src/gemm.jl:318-333), column tiles outer and row tiles inner
 * (:313), software prefetch of A `freq` = 7 columns ahead (src/memory_management.jl:204-237).
 * Remainder rows and columns, which jmul! leaves unwritten (src/gemm.jl:340-345), use the
 * scalar chain here.  Per element the operation order equals chain_f64, so results are
 * bit-identical to or_gemm_f64 whatever the tile.  Threads split the column tiles (the
 * reference is single-threaded; nthreads = 1 is the faithful configuration).
 *
 * Tiles instantiated (rows x cols): f64 40x5 (AVX-512: 8 lanes, 32 registers), 12x4 (AVX2:
 * 4 lanes, 16 registers), 10x5 (128-bit NEON: 2 lanes, 32 registers), 20x5 (4 lanes, 32
 * registers), 16x14 (the one tile of the reference's 16x32x14 benchmark, test/runtests.jl:103-116),
 * 8x6; f32 80x5, 24x4, 20x5, 40x5, 16x14.
 */
/* SIMD width of the host's register file (bytes), the vector type of the tile's columns. */
#if defined(__AVX512F__)
#define OR_VB 64
#elif defined(__AVX2__)
#define OR_VB 32
#else
#define OR_VB 16
#endif
typedef double or_vd __attribute__((vector_size(OR_VB)));
typedef float or_vf __attribute__((vector_size(OR_VB)));

/* One TR x TC tile over the whole K (src/gemm.jl:318-333).  When TR is a multiple of the SIMD
 * width the tile's columns are held as GCC vectors (portable vector extensions, no intrinsics)
 * so that the accumulators stay in registers as the reference's Vec tiles do; acc + a * x is
 * contracted to one fused multiply-add (fp-contract=fast is enabled for these functions only,
 * and no other product meets an add in them), the first step a plain rounded product.  The
 * bit-exact tests against the scalar chain check that every step fused.  Other tiles use
 * scalar fma() loops. */
#define OR_TILED(NAME, T, VT, FMA, TR, TC)                                                          \
  __attribute__((optimize("fp-contract=fast"))) static void NAME##_tile(                          \
      i64 K, const T* pa, i64 lda, const T* pb, i64 ldb, T* pc, i64 ldc) {                          \
    enum { L = OR_VB / (int)sizeof(T), NV = ((TR) % (OR_VB / (int)sizeof(T)) == 0) ? (TR) / (OR_VB / (int)sizeof(T)) : 0 }; \
    if (NV > 0 && K > 0) {                                                                          \
      VT acc[TC][NV > 0 ? NV : 1];                                                                  \
      _Pragma("GCC unroll 32")                                                                      \
      for (int c = 0; c < (TC); ++c) {                                                              \
        const VT x = (VT){0} + pb[c * ldb];                                                         \
        _Pragma("GCC unroll 32")                                                                    \
        for (int v = 0; v < NV; ++v) {                                                              \
          VT a;                                                                                     \
          memcpy(&a, pa + v * L, sizeof(a));                                                        \
          acc[c][v] = a * x;                                                                        \
        }                                                                                           \
      }                                                                                             \
      for (i64 k = 1; k < K; ++k) {                                                                 \
        const T* ak = pa + k * lda;                                                                 \
        __builtin_prefetch(ak + 7 * lda, 0, 3);                                                     \
        VT av[NV > 0 ? NV : 1];                                                                     \
        _Pragma("GCC unroll 32")                                                                    \
        for (int v = 0; v < NV; ++v) memcpy(&av[v], ak + v * L, sizeof(VT));                        \
        _Pragma("GCC unroll 32")                                                                    \
        for (int c = 0; c < (TC); ++c) {                                                            \
          const VT x = (VT){0} + pb[k + c * ldb];                                                   \
          _Pragma("GCC unroll 32")                                                                  \
          for (int v = 0; v < NV; ++v) acc[c][v] = acc[c][v] + av[v] * x;                           \
        }                                                                                           \
      }                                                                                             \
      _Pragma("GCC unroll 32")                                                                      \
      for (int c = 0; c < (TC); ++c)                                                                \
        _Pragma("GCC unroll 32")                                                                    \
        for (int v = 0; v < NV; ++v) memcpy(pc + v * L + c * ldc, &acc[c][v], sizeof(VT));          \
      return;                                                                                       \
    }                                                                                               \
    T acc[TC][TR];                                                                                  \
    if (K == 0) {                                                                                   \
      for (int c = 0; c < (TC); ++c) for (int r = 0; r < (TR); ++r) acc[c][r] = (T)0;               \
    } else {                                                                                        \
      for (int c = 0; c < (TC); ++c) {                                                              \
        const T x = pb[c * ldb];                                                                    \
        for (int r = 0; r < (TR); ++r) acc[c][r] = pa[r] * x;                                       \
      }                                                                                             \
      for (i64 k = 1; k < K; ++k) {                                                                 \
        const T* ak = pa + k * lda;                                                                 \
        __builtin_prefetch(ak + 7 * lda, 0, 3);                                                     \
        T av[TR];                                                                                   \
        for (int r = 0; r < (TR); ++r) av[r] = ak[r];                                               \
        for (int c = 0; c < (TC); ++c) {                                                            \
          const T x = pb[k + c * ldb];                                                              \
          for (int r = 0; r < (TR); ++r) acc[c][r] = FMA(av[r], x, acc[c][r]);                      \
        }                                                                                           \
      }                                                                                             \
    }                                                                                               \
    for (int c = 0; c < (TC); ++c)                                                                  \
      for (int r = 0; r < (TR); ++r) pc[r + c * ldc] = acc[c][r];                                   \
  }                                                                                                 \
  static void NAME(i64 M, i64 N, i64 K, const T* A, i64 lda, const T* B, i64 ldb, T* C, i64 ldc,    \
                   int nthreads, T (*chain)(int, int, i64, i64, i64, const T*, i64, const T*, i64)) {  \
    const i64 col_chunks = N / (TC), row_chunks = M / (TR);                                         \
    /* one thread: no parallel region (its fork/join costs more than a small product) */            \
    _Pragma("omp parallel for schedule(dynamic, 1) num_threads(nthreads > 1 ? nthreads : 1) if(nthreads > 1)") \
    for (i64 cc = 0; cc < col_chunks; ++cc) {                                                       \
      for (i64 rc = 0; rc < row_chunks; ++rc)                                                       \
        NAME##_tile(K, A + rc * (TR), lda, B + cc * (TC) * ldb, ldb, C + rc * (TR) + cc * (TC) * ldc, ldc); \
      for (i64 i = row_chunks * (TR); i < M; ++i)                                                   \
        for (int c = 0; c < (TC); ++c)                                                              \
          C[i + (cc * (TC) + c) * ldc] = chain(0, 0, i, cc * (TC) + c, K, A, lda, B, ldb);          \
    }                                                                                               \
    for (i64 j = col_chunks * (TC); j < N; ++j)                                                     \
      for (i64 i = 0; i < M; ++i) C[i + j * ldc] = chain(0, 0, i, j, K, A, lda, B, ldb);            \
    (void)nthreads;                                                                                 \
  }

OR_TILED(tiled_f64_40x5, double, or_vd, fma, 40, 5)
OR_TILED(tiled_f64_12x4, double, or_vd, fma, 12, 4)
OR_TILED(tiled_f64_10x5, double, or_vd, fma, 10, 5)
OR_TILED(tiled_f64_20x5, double, or_vd, fma, 20, 5)
OR_TILED(tiled_f64_16x14, double, or_vd, fma, 16, 14)
OR_TILED(tiled_f64_8x6, double, or_vd, fma, 8, 6)
OR_TILED(tiled_f32_80x5, float, or_vf, fmaf, 80, 5)
OR_TILED(tiled_f32_24x4, float, or_vf, fmaf, 24, 4)
OR_TILED(tiled_f32_20x5, float, or_vf, fmaf, 20, 5)
OR_TILED(tiled_f32_40x5, float, or_vf, fmaf, 40, 5)
OR_TILED(tiled_f32_16x14, float, or_vf, fmaf, 16, 14)

/* pick_kernel_size (src/kernel_structure.jl:76-99) for elements of t_size bytes in a file of
 * reg_count registers of reg_bytes: grow the rows one register of A at a time (a_loads), give
 * the tile the columns the remaining registers hold (one register kept for the broadcast of
 * X), and stop when the tile's elements per loaded register stop increasing.  Returns the
 * elements per register; rows and cols of the tile through the pointers. */
int or_pick_kernel_size(int t_size, int reg_bytes, int reg_count, int* rows, int* cols) {
  const int epr = reg_bytes / t_size;
  const int lines = (epr * reg_count + epr - 1) / epr;
  int best_r = 0, best_c = 0;
  double best = -1.0 / 0.0;
  for (int a = 1; a <= lines; ++a) {
    const int r = a * epr, c = (reg_count - a - 1) / a;
    const double ratio = (double)(r * c) / (double)(c + a);
    if (ratio < best) break;
    best = ratio;
    best_r = r;
    best_c = c;
  }
  *rows = best_r;
  *cols = best_c;
  return epr;
}

/* Tiled jmul! with a TR x TC tile chosen by the caller; returns -1 for a tile that is not
 * instantiated (nothing is written then). */
int or_jmul_tiled_rc_f64(int tr, int tc, i64 M, i64 N, i64 K, const double* A, i64 lda, const double* B, i64 ldb,
                         double* C, i64 ldc, int nthreads) {
#define OR_CASE(R, C_, FN) \
  if (tr == (R) && tc == (C_)) { FN(M, N, K, A, lda, B, ldb, C, ldc, nthreads, chain_f64); return 0; }
  OR_CASE(40, 5, tiled_f64_40x5) OR_CASE(12, 4, tiled_f64_12x4) OR_CASE(10, 5, tiled_f64_10x5)
  OR_CASE(20, 5, tiled_f64_20x5) OR_CASE(16, 14, tiled_f64_16x14) OR_CASE(8, 6, tiled_f64_8x6)
#undef OR_CASE
  return -1;
}

int or_jmul_tiled_rc_f32(int tr, int tc, i64 M, i64 N, i64 K, const float* A, i64 lda, const float* B, i64 ldb,
                         float* C, i64 ldc, int nthreads) {
#define OR_CASE(R, C_, FN) \
  if (tr == (R) && tc == (C_)) { FN(M, N, K, A, lda, B, ldb, C, ldc, nthreads, chain_f32); return 0; }
  OR_CASE(80, 5, tiled_f32_80x5) OR_CASE(24, 4, tiled_f32_24x4) OR_CASE(20, 5, tiled_f32_20x5)
  OR_CASE(40, 5, tiled_f32_40x5) OR_CASE(16, 14, tiled_f32_16x14)
#undef OR_CASE
  return -1;
}

/* Minimum time in ns of one single-threaded tiled jmul! call (M x N x K, f64, tile tr x tc),
 * over `batches` batches of `reps` back-to-back calls on the same operands (the statistic
 * BenchmarkTools reports as the minimum; test/runtests.jl:111-116).  -1 for a tile that is
 * not instantiated. */
double or_time_jmul_tiled_f64(int tr, int tc, i64 M, i64 N, i64 K, const double* A, const double* B, double* C,
                              int reps, int batches) {
  double best = -1.0;
  for (int b = 0; b < batches; ++b) {
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (int r = 0; r < reps; ++r)
      if (or_jmul_tiled_rc_f64(tr, tc, M, N, K, A, M, B, K, C, M, 1)) return -1.0;
    clock_gettime(CLOCK_MONOTONIC, &t1);
    const double ns = ((double)(t1.tv_sec - t0.tv_sec) * 1e9 + (double)(t1.tv_nsec - t0.tv_nsec)) / reps;
    if (best < 0 || ns < best) best = ns;
  }
  return best;
}

/* ------------------------------------------------------------ near-exact sampled dots */
/*
 * Dot2 of Ogita, Rump and Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 26
 * (2005), Algorithm 5.3: TwoProduct (via fma) and TwoSum give the dot product as if
 * computed in twice the working precision.  Used for the componentwise error metric on
 * sampled entries at sizes where the full oracle is too slow.  For each sample s the
 * output is hi[s] + lo[s] (a double-double) and absdot[s] = sum_k |a_ik| |b_kj| (rounded).
 */
void or_dot2_entries(int ta, int tb, i64 K, const double* A, i64 lda, const double* B, i64 ldb,
                     i64 nsamp, const i64* rows, const i64* cols, double* hi, double* lo,
                     double* absdot, int nthreads) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
#endif
  for (i64 s = 0; s < nsamp; ++s) {
    const i64 i = rows[s], j = cols[s];
    double p = 0.0, q = 0.0, ab = 0.0;
    for (i64 k = 0; k < K; ++k) {
      const double a = A[AIDX(ta, i, k, lda)], b = B[BIDX(tb, k, j, ldb)];
      const double h = a * b;
      const double r = fma(a, b, -h);         /* TwoProduct error term */
      const double t = p + h;                 /* TwoSum(p, h) */
      const double z = t - p;
      const double e = (p - (t - z)) + (h - z);
      p = t;
      q += e + r;
      ab += fabs(a) * fabs(b);
    }
    hi[s] = p + q;
    lo[s] = q - (hi[s] - p);
    absdot[s] = ab;
  }
  (void)nthreads;
}

/*
 * The same sampled entries accumulated in IEEE binary128 (113-bit significand): every
 * product of two doubles is exact in it, and each addition rounds at 2^-113 relative, so
 * |error| <= K 2^-113 sum_k |a_ik b_kj| — an independent near-exact reference next to Dot2.
 * binary128 is __float128 on x86-64 and long double on AArch64 (both software-emulated by
 * libgcc).  Outputs hi[s] + lo[s] (the quad sum rounded to a double-double).
 */
#if defined(__aarch64__)
typedef long double or_quad;
#else
typedef __float128 or_quad;
#endif
void or_quad_entries(int ta, int tb, i64 K, const double* A, i64 lda, const double* B, i64 ldb, i64 nsamp,
                     const i64* rows, const i64* cols, double* hi, double* lo, int nthreads) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
#endif
  for (i64 s = 0; s < nsamp; ++s) {
    const i64 i = rows[s], j = cols[s];
    or_quad acc = 0;
    for (i64 k = 0; k < K; ++k) acc += (or_quad)A[AIDX(ta, i, k, lda)] * (or_quad)B[BIDX(tb, k, j, ldb)];
    const double h = (double)acc;
    hi[s] = h;
    lo[s] = (double)(acc - (or_quad)h);
  }
  (void)nthreads;
}

int or_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* out[i] = fma(a[i], b[i], c[i]) with one rounding (helper for restating fused epilogues). */
void or_fma_array(i64 n, const double* a, const double* b, const double* c, double* out) {
  for (i64 i = 0; i < n; ++i) out[i] = fma(a[i], b[i], c[i]);
}

/* jmul!'s chain (with the alpha/beta extension) for sampled entries only, so that the
 * exact reference value of any element of a large product is cheap to obtain. */
void or_chain_entries_f64(int ta, int tb, i64 K, double alpha, const double* A, i64 lda,
                          const double* B, i64 ldb, double beta, const double* C0, i64 ldc,
                          i64 nsamp, const i64* rows, const i64* cols, double* out, int nthreads) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
#endif
  for (i64 s = 0; s < nsamp; ++s) {
    const i64 i = rows[s], j = cols[s];
    if (alpha == 0.0) { out[s] = (beta == 0.0) ? 0.0 : beta * C0[i + j * ldc]; continue; }
    const double acc = chain_f64(ta, tb, i, j, K, A, lda, B, ldb);
    out[s] = (beta == 0.0) ? alpha * acc : fma(alpha, acc, beta * C0[i + j * ldc]);
  }
  (void)nthreads;
}
void or_chain_entries_f32(int ta, int tb, i64 K, float alpha, const float* A, i64 lda,
                          const float* B, i64 ldb, float beta, const float* C0, i64 ldc,
                          i64 nsamp, const i64* rows, const i64* cols, float* out, int nthreads) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
#endif
  for (i64 s = 0; s < nsamp; ++s) {
    const i64 i = rows[s], j = cols[s];
    if (alpha == 0.0f) { out[s] = (beta == 0.0f) ? 0.0f : beta * C0[i + j * ldc]; continue; }
    const float acc = chain_f32(ta, tb, i, j, K, A, lda, B, ldb);
    out[s] = (beta == 0.0f) ? alpha * acc : fmaf(alpha, acc, beta * C0[i + j * ldc]);
  }
  (void)nthreads;
}
