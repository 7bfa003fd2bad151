/*
 * gbblas — GB300 (sm_103a) GEMM library behind jBLAS.jl's blocked matrix-multiply API.
 *
 * The C ABI below is the drop-in boundary: plain pointers, 64-bit sizes, no CUDA or
 * torch types.  Every matrix pointer is a DEVICE pointer to column-major storage
 * (the layout jBLAS's MMatrix uses, src/gemm.jl:3-11).  `stream` is a cudaStream_t
 * passed as void* (NULL = the legacy default stream).  All calls are stream-ordered:
 * they enqueue work and return; results are valid once the stream reaches that point.
 * Every entry point returns GB_OK (0) or a negative gb_status_t; gb_status_string()
 * gives a message.  Calls are thread-safe as long as concurrent calls use different
 * streams or do not share output buffers.
 *
 * Reference interface each call replaces (paths relative to the jBLAS.jl tree):
 *   gb_jmul_f64 / gb_jmul_f32   jmul!(D, A, X)                src/gemm.jl:244-348
 *   gb_gemm_f64 / gb_gemm_f32   jmul! generalised to BLAS-3  src/gemm.jl:244 (D = A*X,
 *                               alpha/beta and transposes are extensions; the kernel!
 *                               pointer API src/kernels.jl:239 is its D += A*X form)
 *   gb_gemm_grouped_f64/_f32    many independent kernel!/fastmul! products
 *                               src/kernels.jl:202-208, 239 (one launch for all)
 *   gb_gemm_adjoint_f32         no reference counterpart (the rrule of gemm!)
 *   gb_plan_*                   blocking_structure / pick_kernel_size / BLASOptions
 *                               src/memory_management.jl:78-177,
 *                               src/kernel_structure.jl:76-99, src/blas_options.jl:2-7
 */
#ifndef GBBLAS_H
#define GBBLAS_H

#include <stddef.h>
#include <stdint.h>

/* Exported entry points: the library is built with hidden default visibility, so these
 * declarations are its whole dynamic symbol table. */
#if defined(__GNUC__)
#define GB_API __attribute__((visibility("default")))
#else
#define GB_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define GBBLAS_VERSION 100 /* 1.0.0 */

typedef enum {
  GB_OK = 0,
  GB_ERR_INVALID_VALUE = -1,   /* a size, leading dimension, flag or pointer is invalid */
  GB_ERR_UNSUPPORTED = -2,     /* valid request this GPU / build cannot serve */
  GB_ERR_PIPELINE_TIMEOUT = -3,/* a bounded on-device wait expired; the kernel exited */
  GB_ERR_CUDA = -4,            /* a CUDA runtime/driver call failed */
  GB_ERR_ALLOC = -5,           /* device workspace allocation failed */
  GB_ERR_NO_DEVICE = -6        /* no usable sm_103 device is current */
} gb_status_t;

/* Arithmetic mode of gb_gemm_f64 (NATIVE, OZAKI_*) and gb_gemm_f32_ex (NATIVE, BF16X*). */
typedef enum {
  GB_MODE_NATIVE = 0,     /* FP64 FMA chain on the CUDA cores, jBLAS's per-element order */
  GB_MODE_OZAKI_BF16 = 1, /* FP64-accurate emulation: BF16 slices on tcgen05, exact FP32 sums */
  GB_MODE_OZAKI_INT8 = 2, /* INT8 slices: GB_ERR_UNSUPPORTED on sm_103a (no tcgen05 kind::i8) */
  GB_MODE_OZAKI_CRT = 3,  /* FP64-accurate emulation: exact integer product from BF16 residues
                             modulo pairwise coprime moduli (Chinese remainder theorem) */
  GB_MODE_BF16X3 = 4,     /* FP32 on tcgen05: two BF16 terms per value, three term products */
  GB_MODE_BF16X6 = 5      /* FP32 on tcgen05: three BF16 terms per value, six term products */
} gb_mode_t;

GB_API const char* gb_status_string(int status);
GB_API int gb_version(void);

/* Bounded-wait limit (nanoseconds) for every on-device pipeline wait; 0 restores the
 * default (4 s).  A wait that expires makes the kernel exit and the call report
 * GB_ERR_PIPELINE_TIMEOUT on a later gb_check_status(). */
GB_API int gb_set_wait_limit_ns(uint64_t ns);

/* Normwise tolerance the automatic Ozaki slice or moduli count must meet (slices = 0); 0 restores
 * the default 2^-50. */
GB_API int gb_set_ozaki_tolerance(double tol);

/* Engine override for the tensor-core products (slices, FP32 term modes, adjoint): 0 = the
 * engine of the tuning table (gb_set_tc_tuning; CTA pairs by default), 1 = one CTA per
 * 128 x 256 tile, 2 = CTA pairs on 256 x 256 tiles (tcgen05 cta_group::2, half of B per SM).
 * Ozaki results are identical under both engines.  The CRT mode always runs on CTA pairs. */
GB_API int gb_set_tc_engine(int engine);

/* ------------------------------------------------------------------ tensor-core tuning */
/* Launch configuration of the tensor-core engine per kind of product and output-size class:
 * the GPU counterpart of jBLAS's micro-tile choice and block options (pick_kernel_size,
 * src/kernel_structure.jl:76-99; BLASOptions, src/blas_options.jl:2-7), chosen by measurement
 * (gb_autotune_tc) instead of a register-count formula.
 *   engine     1 = one CTA per 128 x 256 output tile (tcgen05 cta_group::1),
 *              2 = a CTA pair per 256 x 256 tile (cta_group::2, each SM loads half of B);
 *              the CRT mode runs on pairs only
 *   band       output-tile rows per band of the tile raster (1..64; tiles of a band share their
 *              A rows in L2)
 *   tma_store  FP32 outputs (GB_TC_F32, GB_TC_ADJOINT) on the pair engine: 1 = C staged in
 *              shared memory and written by TMA stores (beta = 0), 0 = direct stores
 *   panels     GB_TC_OZAKI_CRT only (0 elsewhere): C in blocks — 0 or 1: one; 2: two equal
 *              column panels; 3: three column panels, a narrow first one, a wide middle one and
 *              a last one twice the first's width where that adds no round of 256 x 256 tiles
 *              over the SM pairs to one launch's, else three equal panels where those add
 *              none, else two; 4: 2 x 2 blocks (column panels when M <= 256); at most one per
 *              256 columns.  The residue products of block b run on a high-priority stream of the
 *              library while the caller's stream splits the operand panels of block b + 1 and
 *              reconstructs block b - 1 (and, before the first products, B's statistics and
 *              first panel split run there beside A's).  Under stream capture a call uses one
 *              block.
 *              Results do not depend on it.
 * Size classes by max(M, N): 0 up to 2048, 1 up to 8192, 2 beyond.  gb_set_tc_engine, when set,
 * overrides the engine of every kind. */
typedef enum { GB_TC_OZAKI_SLICES = 0, GB_TC_OZAKI_CRT = 1, GB_TC_F32 = 2, GB_TC_ADJOINT = 3, GB_TC_KINDS = 4 } gb_tc_kind_t;
#define GB_TC_SIZE_CLASSES 3
typedef struct {
  int32_t engine;
  int32_t band;
  int32_t tma_store;
  int32_t panels;
} gb_tc_tuning_t;
GB_API int gb_tc_size_class(int64_t M, int64_t N);
GB_API int gb_tc_default_tuning(int kind, int size_class, gb_tc_tuning_t* out);
GB_API int gb_get_tc_tuning(int kind, int size_class, gb_tc_tuning_t* out);
/* Installs a tuning (NULL = the default) for later calls of that kind and class; an invalid
 * combination gives GB_ERR_INVALID_VALUE. */
GB_API int gb_set_tc_tuning(int kind, int size_class, const gb_tc_tuning_t* tuning);
/* Times every candidate (engines, bands 2..32 pair tiles / 4..64 single tiles, TMA stores where
 * they apply, 1..4 CRT blocks) on seeded synthetic M x N x K operands of the kind (slices: 8 digit slices; CRT:
 * 15 moduli; FP32: BF16X3) with `reps` timed calls after a warm-up, and returns the fastest in
 * `out` (best_ms: its time per call; may be NULL).  The installed tuning is left as it was; the
 * caller installs the result with gb_set_tc_tuning.  Allocates its operands, synchronises
 * `stream`, and changes the engine override and the class's tuning while it runs: make no other
 * tensor-core calls meanwhile. */
GB_API int gb_autotune_tc(int kind, int64_t M, int64_t N, int64_t K, int reps, gb_tc_tuning_t* out, float* best_ms,
                          void* stream);

/* K chunking used by OZAKI calls with an explicit slice count: K is cut into at least
 * `min_chunks` exact accumulation chunks (shorter chunks allow wider digits, at the cost
 * of more accumulator drains); 0 or 1 restores the default (one chunk up to K = 65536).
 * slices = 0 ignores it and chooses slices and chunking together. */
GB_API int gb_set_ozaki_min_chunks(int min_chunks);

/* Measured FMA-pipe peaks of the current device in TFLOP/s (either pointer may be NULL): a
 * register-only loop of independent FMA chains on every SM, FP64 (DFMA) and FP32 (FFMA), timed
 * with CUDA events.  The CUDA-core counterpart of jBLAS's machine constants (deps/build.jl:26-34);
 * it takes a few milliseconds and synchronises the device. */
GB_API int gb_measure_fma_peaks(double* fp64_tflops, double* fp32_tflops);

/* Returns the current device's cached workspace memory to the CUDA driver (synchronises the
 * device).  Workspace is otherwise kept between calls. */
GB_API int gb_release_workspace(void);

/* Reads and clears the device-side status word written by timed-out waits (synchronises
 * `stream`).  There is one status word per device, shared by every call on that device from
 * every stream and thread: the first expired wait since the last check is reported by
 * whichever check comes next, and the read and the clear are one atomic step, so a report is
 * never lost between them. */
GB_API int gb_check_status(void* stream);

/* ------------------------------------------------------------------ tracing */
/* Kernel kinds counted and timed by the tracing layer. */
typedef enum {
  GB_KERNEL_OZAKI_STATS = 0,
  GB_KERNEL_OZAKI_SPLIT = 1,
  GB_KERNEL_OZAKI_SLICE_MMA = 2,
  GB_KERNEL_NATIVE_GEMM = 3,
  GB_KERNEL_SCALE_C = 4,
  GB_KERNEL_GROUPED_GEMM = 5,
  GB_KERNEL_ADJOINT_SPLIT = 6,
  GB_KERNEL_ADJOINT_MMA = 7,
  GB_KERNEL_OZAKI_COMBINE = 8,   /* CRT reconstruction of the residue products */
  GB_KERNEL_SEMIRING_GEMM = 9,
  GB_KERNEL_F32_SPLIT = 10,      /* BF16 term planes of gb_gemm_f32_ex's tensor-core modes */
  GB_KERNEL_F32_MMA = 11,        /* their term products on tcgen05 */
  GB_KERNEL_KINDS = 16
} gb_kernel_kind_t;
GB_API const char* gb_kernel_kind_name(int kind);
/* Launches of each kernel kind since the library was loaded (counts[0..n)). */
GB_API int gb_launch_counts(long long* counts, int n);
/* Between start and stop, every launch is bracketed by CUDA events on its stream; stop
 * synchronises those events and returns the summed milliseconds and launch count of
 * each kind (ms[0..n), launches[0..n); either may be NULL). */
GB_API int gb_profile_start(void);
GB_API int gb_profile_stop(double* ms, long long* launches, int n);

/* ------------------------------------------------------------------ jmul! proper */
/* D (M x P) = A (M x N) * X (N x P), contraction over N, leading dimensions M, N, M
 * exactly as an MMatrix (src/gemm.jl:244).  Per element d = a1*x1; d = fma(ak, xk, d)
 * for k = 2..N in order: results are bit-identical to jmul!'s arithmetic, and every
 * element is written (jmul! leaves remainder tiles unwritten, src/gemm.jl:340-345). */
GB_API int gb_jmul_f64(double* D, const double* A, const double* X, int64_t M, int64_t N, int64_t P,
                void* stream);
GB_API int gb_jmul_f32(float* D, const float* A, const float* X, int64_t M, int64_t N, int64_t P,
                void* stream);

/* ------------------------------------------------------------------ kernel! (pointer form) */
/* jBLAS's pointer-level micro-kernels on device pointers, with their argument meaning.
 * kernel!(pD, pA, pX, Kernel{Mk,Pk,stride_AD,stride_X,N}) (src/kernels.jl:212-239):
 *   D (Mk x Pk) += A (Mk x N) * X (N x Pk), A and D with leading dimension stride_AD, X with
 *   stride_X; per element d = fma(a_n, x_n, d) for n = 1..N in order, starting from D's value
 *   (bit-identical to the reference's vmuladd chain).
 * init != 0: initkernel! (src/kernels.jl:240-273): D = A * X with d = a_1 * x_1, then the same
 *   chain (D is not read).
 * Extensions: any Mk (the reference requires a multiple of the SIMD width, src/kernels.jl:219)
 * and any size; N = 0 leaves D unchanged (init: D = 0). */
GB_API int gb_kernel_f64(double* pD, const double* pA, const double* pX, int64_t Mk, int64_t Pk, int64_t stride_AD,
                         int64_t stride_X, int64_t N, int init, void* stream);
GB_API int gb_kernel_f32(float* pD, const float* pA, const float* pX, int64_t Mk, int64_t Pk, int64_t stride_AD,
                         int64_t stride_X, int64_t N, int init, void* stream);

/* ------------------------------------------------------------------ BLAS-3 GEMM */
/* C = alpha*op(A)*op(B) + beta*C; op(X) = X (trans = 0) or X^T (trans = 1).
 * op(A) is M x K, op(B) is K x N, C is M x N; lda >= rows of A as stored, etc.
 * beta == 0: C is not read (NaN in C is overwritten).  alpha == 0 or K == 0:
 * C = beta*C and A, B are not read.
 * mode GB_MODE_NATIVE: per element acc = fma chain in k order (as jmul!), then
 *   C = alpha*acc (beta == 0) or fma(alpha, acc, beta*C).
 * mode GB_MODE_OZAKI_BF16: A and B are split into `slices` BF16 digit planes with
 *   per-row / per-column power-of-two scaling (slices = 0 picks the count that meets
 *   the library's default tolerance, 2^-50 normwise); slice products run on tcgen05
 *   with exact FP32 accumulation and are recombined in FP64.  Rows of A or columns of
 *   B holding Inf/NaN give NaN in the outputs they touch.
 * mode GB_MODE_OZAKI_CRT: rows of op(A) and columns of op(B) are scaled by powers of two
 *   and rounded (half away from zero) to integers of t bits; their product is formed
 *   exactly from `slices` residue products (one BF16 tcgen05 GEMM per modulus, moduli
 *   <= 253, exact FP32 sums) and the Chinese remainder theorem, then rounded once to
 *   FP64 and rescaled.  slices = number of moduli (1..20; t follows from K, see
 *   gb_plan_ozaki_crt); slices = 0 picks the fewest moduli whose bound meets the
 *   library tolerance (t then also uses the operands' row sums).  Inf/NaN as for BF16.
 * err_bound_out (host pointer, may be NULL): for OZAKI_BF16 / OZAKI_CRT, an a-priori bound
 *   on ||C - C_exact||_F / (|alpha| ||A||_F ||B||_F) from the truncation of the operands;
 *   the call then synchronises `stream` to read it.  Without it an OZAKI_CRT call never
 *   synchronises (its plan is chosen on the device) and can be captured in a CUDA graph;
 *   OZAKI_BF16 with slices = 0 synchronises once to read the split statistics.  For NATIVE it
 *   receives the standard bound K*u/(1-K*u) (u = 2^-53) of the same quantity. */
GB_API int gb_gemm_f64(int transA, int transB, int64_t M, int64_t N, int64_t K, double alpha,
                const double* A, int64_t lda, const double* B, int64_t ldb, double beta,
                double* C, int64_t ldc, int mode, int slices, double* err_bound_out,
                void* stream);
GB_API int gb_gemm_f32(int transA, int transB, int64_t M, int64_t N, int64_t K, float alpha,
                const float* A, int64_t lda, const float* B, int64_t ldb, float beta,
                float* C, int64_t ldc, void* stream);
/* gb_gemm_f32 with an arithmetic mode (gb_gemm_f32 is mode GB_MODE_NATIVE: the jmul! FMA chain,
 * bit for bit).  The tensor-core modes have no reference counterpart; they give up jmul!'s
 * per-element order for tcgen05 throughput.  Every FP32 value is split into BF16 terms
 * (t_0 = bf16(x), t_1 = bf16(x - t_0), t_2 = bf16(x - t_0 - t_1)) and the term products with
 * p + q below the term count are accumulated in FP32 on the tensor cores:
 *   GB_MODE_BF16X3  2 terms, 3 products; per element |C - C_exact| <= about
 *                   (2^-15 + K 2^-24) |alpha| (|op(A)| |op(B)|)_ij  (+ beta C rounding)
 *   GB_MODE_BF16X6  3 terms, 6 products; about (2^-21 + K 2^-24) |alpha| (|op(A)| |op(B)|)_ij,
 *                   FP32-level accuracy
 * Workspace (the term planes, (terms) x (M + N) x K BF16) comes from the library pool.  Other
 * modes give GB_ERR_INVALID_VALUE.  Arguments, transposes, alpha/beta rules as gb_gemm_f32. */
GB_API int gb_gemm_f32_ex(int transA, int transB, int64_t M, int64_t N, int64_t K, float alpha,
                          const float* A, int64_t lda, const float* B, int64_t ldb, float beta,
                          float* C, int64_t ldc, int mode, void* stream);

/* ------------------------------------------------------------------ host buffers */
/* The same products on HOST buffers, for callers whose matrices live in host memory as the
 * reference's MMatrix operands do (pageable or pinned; device pointers work too, through
 * unified addressing).  The call uploads op(A), op(B) (and C when beta != 0) into library
 * workspace, runs gb_gemm_* on `stream` with the same mode and arguments, downloads C and
 * returns once `stream` has finished: results are those of the device call, bit for bit.
 * With a pinned (page-locked) C, a CRT call in column panels copies each panel to C on a
 * stream of the library as soon as it is reconstructed, beside the later panels' products;
 * three panels are then two halves and a narrow last panel (the tuning's `panels` = 3).
 * A bounded on-device wait that expired is reported as GB_ERR_PIPELINE_TIMEOUT (the status
 * word is read and cleared).  gb_jmul_*_host: jmul!(D, A, X) on host MMatrix-like buffers
 * (leading dimensions M, N, M). */
GB_API int gb_gemm_f64_host(int transA, int transB, int64_t M, int64_t N, int64_t K, double alpha, const double* A,
                            int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc, int mode,
                            int slices, double* err_bound_out, void* stream);
GB_API int gb_gemm_f32_host(int transA, int transB, int64_t M, int64_t N, int64_t K, float alpha, const float* A,
                            int64_t lda, const float* B, int64_t ldb, float beta, float* C, int64_t ldc, void* stream);
GB_API int gb_jmul_f64_host(double* D, const double* A, const double* X, int64_t M, int64_t N, int64_t P,
                            void* stream);
GB_API int gb_jmul_f32_host(float* D, const float* A, const float* X, int64_t M, int64_t N, int64_t P, void* stream);

/* ------------------------------------------------------------------ grouped GEMM */
/* One independent product C = alpha*A*B + beta*C (column-major, no transposes, device
 * pointers; alpha == 0: A, B not read; beta == 0: C not read). */
typedef struct {
  int64_t m, n, k;
  int64_t lda, ldb, ldc;
  const void* A;
  const void* B;
  void* C;
  double alpha, beta;   /* used as float by the f32 entry point */
} gb_problem_t;

/* Tile configuration per size class.  Classes by max(m, n): <=16, <=32, <=64, <=128,
 * <=256, >256.  Configurations (rows x cols of a C tile, 256 threads each):
 *   0: 16x16  1: 32x32  2: 64x32  3: 64x64                     (f64 and f32)
 *   4: 128x64  5: 128x128  6: 32x64  7: 64x128  8: 128x32  9: 32x128   (f32 only)
 *   GB_GROUPED_AUTO: chosen per problem from its m, n and k by a cost model (padding of the
 *   tiles against the FMA efficiency of their register tiles; the FP32 default)
 * This replaces jBLAS's fixed BLASOptions(m_k, p_k) (src/blas_options.jl:2-7). */
#define GB_GROUPED_CLASSES 6
#define GB_GROUPED_CONFIGS 10
#define GB_GROUPED_AUTO 31
typedef struct {
  int32_t config[GB_GROUPED_CLASSES];
} gb_grouped_tuning_t;

GB_API int gb_grouped_default_tuning(int dtype_bytes, gb_grouped_tuning_t* out);
/* Device workspace a grouped call over `count` problems needs (tile prefix sums and the schedule
 * order: 8 (count + 1 + (count + 1) / 2) bytes). */
GB_API size_t gb_grouped_workspace_size(int count);
/* All `count` products (table `problems` in DEVICE memory) in one persistent launch after
 * a prologue that counts tiles per problem.  tuning NULL = defaults.  workspace NULL =
 * taken from the library's pool; a caller-provided workspace (>= gb_grouped_workspace_size)
 * makes the call allocation-free, e.g. for CUDA-graph capture.  Per element the result
 * equals jmul!'s FMA chain (with the alpha/beta extension of gb_gemm_*).  The table's
 * sizes and pointers are trusted (device memory is not inspected on the host).
 * Reference: many fastmul!/kernel! products, src/kernels.jl:202-208, 239. */
GB_API int gb_gemm_grouped_f64(const gb_problem_t* problems, int count, const gb_grouped_tuning_t* tuning,
                        void* workspace, size_t workspace_bytes, void* stream);
GB_API int gb_gemm_grouped_f32(const gb_problem_t* problems, int count, const gb_grouped_tuning_t* tuning,
                        void* workspace, size_t workspace_bytes, void* stream);
/* Allocation-free grouped FP64 GEMM.  No counterpart in the reference (jBLAS never
 * allocates because it only multiplies static-size arrays on the CPU).  For callers that
 * cannot allocate device memory when they multiply: threads that must not block on the
 * implicit device synchronisation of cudaMalloc/cudaFree (a latency-bound serving loop, a
 * callback running under another library's lock), and hosts whose device memory is
 * entirely owned by another runtime or allocator.  The call's scratch (tile prefix sums and the
 * order in which the problems are scheduled) lives in a file-scope device array of 98,305
 * int64 (768 KiB), which every GPU that loads the library keeps until the process exits.  count above the maximum gives
 * GB_ERR_INVALID_VALUE.  The first call on a device looks the array's device address up
 * (cudaGetSymbolAddress, no allocation); make that first call before any stream capture.
 * Every call shares the one array: calls that overlap on the GPU (other streams, other
 * threads) race and must be serialised by the caller.  Results equal gb_gemm_grouped_f64's.
 * A null or host `problems` table gives GB_ERR_INVALID_VALUE before anything is launched.
 * gb_launch_counts counts its launches; the profiling timers (gb_profile_start/stop) do not
 * time them, because timing would create CUDA events. */
#define GB_GROUPED_NOALLOC_MAX 65536
GB_API int gb_gemm_grouped_f64_noalloc(const gb_problem_t* problems, int count, const gb_grouped_tuning_t* tuning,
                                void* stream);
/* Strided batched GEMM: C_i = alpha A_i B_i + beta C_i for i < count, where A_i = A + i*strideA,
 * B_i = B + i*strideB, C_i = C + i*strideC (strides in elements, >= 0; a stride of 0 shares
 * that operand), each product M x N x K, column-major, no transposes, device pointers; the
 * C_i must not overlap.  The batch form of jBLAS's fastmul!/kernel! on many small static
 * matrices (src/kernels.jl:1-208, 239): per element the jmul! FMA chain (bit-identical, with
 * the alpha/beta extension of gb_gemm_*), run as one grouped persistent launch over a
 * problem table built on the device (table and workspace from the library pool).
 * count <= 2^31 - 1. */
GB_API int gb_gemm_strided_batched_f64(int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t lda,
                                int64_t strideA, const double* B, int64_t ldb, int64_t strideB, double beta,
                                double* C, int64_t ldc, int64_t strideC, int64_t count, void* stream);
GB_API int gb_gemm_strided_batched_f32(int64_t M, int64_t N, int64_t K, float alpha, const float* A, int64_t lda,
                                int64_t strideA, const float* B, int64_t ldb, int64_t strideB, float beta,
                                float* C, int64_t ldc, int64_t strideC, int64_t count, void* stream);

/* ------------------------------------------------------------------ semiring GEMM */
/* C = [C (+)] (+)_k op(A)[i,k] (x) op(B)[k,j] over a semiring ((+), (x)) instead of
 * (+, *).  No counterpart in the reference's code: jBLAS keeps its tuple-SIMD Vec type
 * (src/simd.jl) out of the module with the note "Maybe use that as a fallback for custom
 * number types? Eg, so it works with min-plus algebra?" (src/jBLAS.jl:10).  Same layout,
 * transposes and register-blocked CUDA-core mainloop as gb_gemm_* NATIVE.
 *   (+) = min or max; for floating point a NaN operand is ignored (IEEE minNum/maxNum:
 *         the result is NaN only when every candidate is NaN), and a zero result is
 *         returned as +0.0, so the result does not depend on the K order;
 *   (x) = +, *, min or max, rounded once (round to nearest); int32 + and * wrap modulo 2^32.
 * accumulate = 0: C = (+)_k ...; the empty K gives the identity of (+) (+Inf / -Inf,
 * INT32_MAX / INT32_MIN).  accumulate = 1: C is read and folded in with (+).
 * Errors as gb_gemm_*: GB_ERR_INVALID_VALUE for an unknown semiring or accumulate flag. */
typedef enum {
  GB_SEMIRING_MIN_PLUS = 0,    /* (min, +): shortest paths (tropical) */
  GB_SEMIRING_MAX_PLUS = 1,    /* (max, +): longest / critical paths, log-space Viterbi */
  GB_SEMIRING_MAX_MIN = 2,     /* (max, min): widest (bottleneck) paths */
  GB_SEMIRING_MIN_MAX = 3,     /* (min, max): minimax paths */
  GB_SEMIRING_MAX_TIMES = 4,   /* (max, *): Viterbi on probabilities */
  GB_SEMIRINGS = 5
} gb_semiring_t;
GB_API int gb_gemm_semiring_f64(int semiring, int transA, int transB, int64_t M, int64_t N, int64_t K,
                         const double* A, int64_t lda, const double* B, int64_t ldb, int accumulate,
                         double* C, int64_t ldc, void* stream);
GB_API int gb_gemm_semiring_f32(int semiring, int transA, int transB, int64_t M, int64_t N, int64_t K,
                         const float* A, int64_t lda, const float* B, int64_t ldb, int accumulate,
                         float* C, int64_t ldc, void* stream);
GB_API int gb_gemm_semiring_i32(int semiring, int transA, int transB, int64_t M, int64_t N, int64_t K,
                         const int32_t* A, int64_t lda, const int32_t* B, int64_t ldb, int accumulate,
                         int32_t* C, int64_t ldc, void* stream);
/* Autotuner: times every configuration per size class on the given problems (HOST copy
 * of the table; their C buffers are left untouched, results go to scratch) with `reps`
 * timed repetitions and writes the fastest configuration per class; class_ms (may be
 * NULL) receives the best time per class in ms.  Synchronises `stream`.
 * Reference: pick_kernel_size / blocking_structure, src/kernel_structure.jl:76-99,
 * src/memory_management.jl:78-177. */
GB_API int gb_autotune_grouped(int dtype_bytes, const gb_problem_t* host_problems, int count, int reps,
                        gb_grouped_tuning_t* out, float* class_ms, void* stream);

/* ------------------------------------------------------------------ adjoint */
/* Pullback of C = A*B (A M x K, B K x N, column-major FP32): given dC (M x N),
 *   dA = dC * B^T  (M x K)   and   dB = A^T * dC  (K x N)
 * in one tensor-core launch.  No reference counterpart: it is the rrule of jBLAS's
 * jmul!/gemm! (src/gemm.jl:244).  Products use the 3xBF16 split (x = hi + lo, the
 * lo*lo term dropped) with FP32 accumulation: per element |error| <= about
 * 2^-15 (|dC||B|^T)_ik plus FP32 summation error.  dC is read from memory once. */
GB_API int gb_gemm_adjoint_f32(int64_t M, int64_t N, int64_t K, const float* A, int64_t lda, const float* B,
                        int64_t ldb, const float* dC, int64_t lddc, float* dA, int64_t ldda, float* dB,
                        int64_t lddb, void* stream);

/* Ozaki plan for a problem: slice count, bits per slice and the grouping of slice
 * products that the tensor-core kernel would use (no GPU work). */
typedef struct {
  int32_t slices;        /* digit planes per operand */
  int32_t bits;          /* bits per digit plane (|digit| <= 2^(bits-1)) */
  int32_t k_chunk;       /* K elements per exact FP32 accumulation */
  int32_t products;      /* slice-pair products per K chunk (p + q <= slices + 1) */
  int32_t groups;        /* TMEM accumulation groups drained per output tile */
  double  flops_tensor;  /* BF16 tensor flops the plan issues */
} gb_ozaki_plan_t;
GB_API int gb_plan_ozaki(int64_t M, int64_t N, int64_t K, int slices, gb_ozaki_plan_t* out);
/* CRT plan for `moduli` moduli (1..20): slices = moduli, bits = t (the integer width of
 * the scaled operands: largest t <= 62 with 4 K 2^(2t) <= product of the moduli and
 * K 2^(2t) <= 2^125), k_chunk, products = groups = moduli, flops_tensor.
 * GB_ERR_UNSUPPORTED when no t >= 1 fits. */
GB_API int gb_plan_ozaki_crt(int64_t M, int64_t N, int64_t K, int moduli, gb_ozaki_plan_t* out);
/* Blocks of C of a CRT call on an M x N output (see gb_tc_tuning_t.panels): for the tuning's
 * `panels` value, a device of `sms` SMs (the residue products run one 256 x 256 tile per SM
 * pair at a time) and host_copies = 1 for a host-buffer call with a pinned C, the row
 * boundaries rows[0..*row_blocks] (at most 2 blocks) and column boundaries
 * cols[0..*col_blocks] (at most 4) of the blocks, multiples of 256 but the last.  A call under
 * stream capture runs one block whatever this returns. */
GB_API int gb_crt_blocks(int64_t M, int64_t N, int panels, int sms, int host_copies, int64_t* rows, int* row_blocks,
                         int64_t* cols, int* col_blocks);
/* The plan of the most recent OZAKI (BF16 or CRT) gb_gemm_f64 call made by the calling
 * thread (zeroes before the first), e.g. the slice count an automatic call picked. */
GB_API int gb_last_ozaki_plan(gb_ozaki_plan_t* out);

#ifdef __cplusplus
}
#endif
#endif /* GBBLAS_H */
