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
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
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
 * The jmul! algorithm as the reference generates it: a rows x cols register tile
 * (src/kernel_structure.jl:76-99 pick_kernel_size), the full K reduction held in the
 * tile (src/gemm.jl:318-333), column tiles outer and row tiles inner (:313), software
 * prefetch of A `freq` columns ahead (src/memory_management.jl:204-237, default 7).
 * The tile here is 8 x 6 doubles (16 x 6 floats), the shape pick_kernel_size gives for
 * 32 registers of 4 lanes; remainder tiles use the scalar chain.  Per element the
 * operation order equals chain_f64, so results are bit-identical to or_gemm_f64.
 * Threads split the column tiles (the reference is single-threaded; nthreads = 1 is
 * the faithful configuration).
 */
#define TMR 8
#define TNR 6
#define TMR32 16

void or_jmul_tiled_f64(i64 M, i64 N, i64 K, const double* A, i64 lda, const double* B, i64 ldb,
                       double* C, i64 ldc, int nthreads) {
  const i64 col_chunks = N / TNR, row_chunks = M / TMR;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
#endif
  for (i64 cc = 0; cc < col_chunks; ++cc) {
    for (i64 rc = 0; rc < row_chunks; ++rc) {
      const double* pa = A + rc * TMR;
      const double* pb = B + cc * TNR * ldb;
      double acc[TNR][TMR];
      if (K == 0) {
        for (int c = 0; c < TNR; ++c) for (int r = 0; r < TMR; ++r) acc[c][r] = 0.0;
      } else {
        for (int c = 0; c < TNR; ++c) {
          const double x = pb[c * ldb];
          for (int r = 0; r < TMR; ++r) acc[c][r] = pa[r] * x;
        }
        for (i64 k = 1; k < K; ++k) {
          const double* ak = pa + k * lda;
          __builtin_prefetch(ak + 7 * lda, 0, 3);
          double av[TMR];
          for (int r = 0; r < TMR; ++r) av[r] = ak[r];
          for (int c = 0; c < TNR; ++c) {
            const double x = pb[k + c * ldb];
            for (int r = 0; r < TMR; ++r) acc[c][r] = fma(av[r], x, acc[c][r]);
          }
        }
      }
      for (int c = 0; c < TNR; ++c)
        for (int r = 0; r < TMR; ++r) C[rc * TMR + r + (cc * TNR + c) * ldc] = acc[c][r];
    }
    for (i64 i = row_chunks * TMR; i < M; ++i)
      for (int c = 0; c < TNR; ++c)
        C[i + (cc * TNR + c) * ldc] = chain_f64(0, 0, i, cc * TNR + c, K, A, lda, B, ldb);
  }
  for (i64 j = col_chunks * TNR; j < N; ++j)
    for (i64 i = 0; i < M; ++i) C[i + j * ldc] = chain_f64(0, 0, i, j, K, A, lda, B, ldb);
  (void)nthreads;
}

void or_jmul_tiled_f32(i64 M, i64 N, i64 K, const float* A, i64 lda, const float* B, i64 ldb,
                       float* C, i64 ldc, int nthreads) {
  const i64 col_chunks = N / TNR, row_chunks = M / TMR32;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
#endif
  for (i64 cc = 0; cc < col_chunks; ++cc) {
    for (i64 rc = 0; rc < row_chunks; ++rc) {
      const float* pa = A + rc * TMR32;
      const float* pb = B + cc * TNR * ldb;
      float acc[TNR][TMR32];
      if (K == 0) {
        for (int c = 0; c < TNR; ++c) for (int r = 0; r < TMR32; ++r) acc[c][r] = 0.0f;
      } else {
        for (int c = 0; c < TNR; ++c) {
          const float x = pb[c * ldb];
          for (int r = 0; r < TMR32; ++r) acc[c][r] = pa[r] * x;
        }
        for (i64 k = 1; k < K; ++k) {
          const float* ak = pa + k * lda;
          __builtin_prefetch(ak + 7 * lda, 0, 3);
          float av[TMR32];
          for (int r = 0; r < TMR32; ++r) av[r] = ak[r];
          for (int c = 0; c < TNR; ++c) {
            const float x = pb[k + c * ldb];
            for (int r = 0; r < TMR32; ++r) acc[c][r] = fmaf(av[r], x, acc[c][r]);
          }
        }
      }
      for (int c = 0; c < TNR; ++c)
        for (int r = 0; r < TMR32; ++r) C[rc * TMR32 + r + (cc * TNR + c) * ldc] = acc[c][r];
    }
    for (i64 i = row_chunks * TMR32; i < M; ++i)
      for (int c = 0; c < TNR; ++c)
        C[i + (cc * TNR + c) * ldc] = chain_f32(0, 0, i, cc * TNR + c, K, A, lda, B, ldb);
  }
  for (i64 j = col_chunks * TNR; j < N; ++j)
    for (i64 i = 0; i < M; ++i) C[i + j * ldc] = chain_f32(0, 0, i, j, K, A, lda, B, ldb);
  (void)nthreads;
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
