/*
 * quadblas_gpu.h — C ABI of libquadblas_gpu.so, a GB300 (sm_103a) GPU
 * implementation of QuadBLAS's IEEE binary128 BLAS hot path.
 *
 * Binary128 arguments are `void *` pointers to 16-byte IEEE binary128
 * values (Sleef_quad, __float128, AArch64 long double), little-endian,
 * 16-byte aligned for the device-pointer entry points.
 *
 * Part 1 keeps the reference's C interface signatures
 * (include/quadblas/interface/c_interface.hpp of QuadBLAS 1.0.0) so that
 * existing callers link unchanged.  Part 2 adds binary128 scalars/results,
 * 64-bit sizes and status returns; part 3 adds device-pointer entry points
 * ordered on a caller-given CUDA stream.
 *
 * Semantics shared by all entry points:
 *  - dot, gemv and gemm sums are the exact sum of the exact products,
 *    rounded to binary128 once (round to nearest, ties to even) — except
 *    in the rare case where the exact sum is within about
 *    n * 2^-190 * max|a_i b_i| of a rounding boundary, or where the
 *    Ozaki method is selected for qgemm (then the accuracy is set by the
 *    slice count).  The reference instead
 *    rounds after every FMA; both are within k * 2^-113 * sum|a_i b_i|
 *    of each other.
 *  - gemv/gemm then apply the reference epilogue y = fma(alpha, sum, beta*y)
 *    with one rounding, bit-identical to SLEEF's Sleef_fmaq1_u05.
 *  - axpy is y_i = fma(alpha, x_i, y_i), bit-identical to the reference.
 *  - Increments must be positive.  Column-major ('C'/'c') and transposed
 *    ('T','t','C','c') operands are supported by qgemv (as in the
 *    reference) and by qgemm (the reference ignores transa/transb and
 *    mis-indexes column-major C above 64; this library implements the
 *    intended semantics of the reference's test loops).
 *  - Status codes are the QBLAS_* values below.
 */
#ifndef QUADBLAS_GPU_H
#define QUADBLAS_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  QBLAS_OK = 0,
  QBLAS_ERR_INVALID_VALUE = 1,
  QBLAS_ERR_CUDA = 2,
  QBLAS_ERR_NO_MEMORY = 3,
  QBLAS_ERR_NOT_SUPPORTED = 4,
  QBLAS_ERR_NO_DEVICE = 5,
  QBLAS_ERR_MISALIGNED = 6,
  /* a wait inside an Ozaki qgemm kernel gave up (1 s without progress); the
   * call's C is not valid (NaN, or left unwritten where the reconstruction
   * itself gave up) */
  QBLAS_ERR_TIMEOUT = 7
};

enum { QBLAS_METHOD_AUTO = 0, QBLAS_METHOD_SOFTFLOAT = 1, QBLAS_METHOD_OZAKI = 2 };

/* ---- Part 1: reference-compatible entry points (host pointers) --------- */

/* Replaces quadblas_qdot, c_interface.hpp:21.  Returns the binary128 dot
 * rounded to double (as the reference does). */
double quadblas_qdot(int n, void *x, int incx, void *y, int incy);

/* Replaces quadblas_qnrm2, c_interface.hpp:34: sqrt(dot(x, x)). */
double quadblas_qnrm2(int n, void *x, int incx);

/* Replaces quadblas_qaxpy, c_interface.hpp:47: y = alpha*x + y. */
void quadblas_qaxpy(int n, double alpha, void *x, int incx, void *y, int incy);

/* Replaces quadblas_qgemv, c_interface.hpp:64: y = alpha*op(A)*x + beta*y;
 * layout 'C'/'c' = column-major, else row-major; trans in T/t/C/c swaps
 * m and n and flips the layout (c_interface.hpp:79-85). */
void quadblas_qgemv(char layout, char trans, int m, int n, double alpha, void *A, int lda,
                    void *x, int incx, double beta, void *y, int incy);

/* Replaces quadblas_qgemm, c_interface.hpp:95: C = alpha*op(A)*op(B) + beta*C. */
void quadblas_qgemm(char layout, char transa, char transb, int m, int n, int k, double alpha,
                    void *A, int lda, void *B, int ldb, double beta, void *C, int ldc);

/* Replaces quadblas_set_num_threads / get_num_threads, c_interface.hpp:122,128.
 * Kept for ABI compatibility: the value is recorded and reported, the GPU
 * path has no host thread pool. */
void quadblas_set_num_threads(int num_threads);
int quadblas_get_num_threads(void);

/* Replaces quadblas_get_version, c_interface.hpp:134. */
const char *quadblas_get_version(void);

/* Replaces quadblas_is_aligned, c_interface.hpp:140 (32-byte test). */
int quadblas_is_aligned(const void *ptr);

/* ---- Part 2: binary128 scalars and results, host pointers ------------- */
/* Same operations as part 1 (QuadBLAS::dot/axpy/gemv/gemm,
 * algorithms/level1.hpp:80,190, level2.hpp:85, level3.hpp:215, which the
 * C++ classes of interface/cpp_classes.hpp:66-153 call with binary128
 * scalars); alpha, beta and result point to binary128 values. */
int quadblas_qdot_q(int64_t n, const void *x, int64_t incx, const void *y, int64_t incy,
                    void *result);
int quadblas_qnrm2_q(int64_t n, const void *x, int64_t incx, void *result);
int quadblas_qaxpy_q(int64_t n, const void *alpha, const void *x, int64_t incx, void *y,
                     int64_t incy);
int quadblas_qgemv_q(char layout, char trans, int64_t m, int64_t n, const void *alpha,
                     const void *A, int64_t lda, const void *x, int64_t incx, const void *beta,
                     void *y, int64_t incy);
int quadblas_qgemm_q(char layout, char transa, char transb, int64_t m, int64_t n, int64_t k,
                     const void *alpha, const void *A, int64_t lda, const void *B, int64_t ldb,
                     const void *beta, void *C, int64_t ldc);

/* ---- Part 3: device pointers, ordered on `stream` (a cudaStream_t; NULL
 * is the legacy default stream).  alpha/beta are HOST pointers to
 * binary128 values; d_result is a device pointer.  The calls return after
 * enqueueing the work.  Same operations as part 2; no reference
 * counterpart (the reference is CPU-only). */
int quadblas_qdot_dev(int64_t n, const void *dx, int64_t incx, const void *dy, int64_t incy,
                      void *d_result, void *stream);
int quadblas_qnrm2_dev(int64_t n, const void *dx, int64_t incx, void *d_result, void *stream);
int quadblas_qaxpy_dev(int64_t n, const void *alpha, const void *dx, int64_t incx, void *dy,
                       int64_t incy, void *stream);
int quadblas_qgemv_dev(char layout, char trans, int64_t m, int64_t n, const void *alpha,
                       const void *dA, int64_t lda, const void *dx, int64_t incx,
                       const void *beta, void *dy, int64_t incy, void *stream);
int quadblas_qgemm_dev(char layout, char transa, char transb, int64_t m, int64_t n, int64_t k,
                       const void *alpha, const void *dA, int64_t lda, const void *dB,
                       int64_t ldb, const void *beta, void *dC, int64_t ldc, void *stream);

/* Capacity of quadblas_qdot_dev_noalloc's static scratch, in partial
 * accumulators of 40 bytes (40 KiB, plus 16 KiB for the exact pass). */
#define QBLAS_NOALLOC_MAX_PARTIALS 1024

/* No counterpart in the reference.  Same operation and result as
 * quadblas_qdot_dev, for callers that cannot allocate device memory —
 * programs whose device memory belongs to their own allocator or a fixed
 * memory plan, and latency-sensitive loops that cannot call into the CUDA
 * allocator — so it allocates nothing: its scratch is a static 56 KiB array
 * that the library keeps on every GPU it is loaded on, until exit.  Any n
 * fits on GPUs with up to 256 SMs; a problem that would need more than
 * QBLAS_NOALLOC_MAX_PARTIALS partial accumulators returns
 * QBLAS_ERR_INVALID_VALUE.  The first call on a device looks up the array's
 * address (make that call before any stream capture).  All calls share the
 * array: calls that overlap on the GPU race.  The status is reported by the
 * return value only (quadblas_last_error is not updated). */
int quadblas_qdot_dev_noalloc(int64_t n, const void *dx, int64_t incx, const void *dy,
                              int64_t incy, void *d_result, void *stream);

/* ---- Part 4: batched problems in one persistent launch (no reference
 * counterpart; each problem has the semantics of the single call).
 *   QBLAS_OP_GEMM: C = alpha*op(A)*op(B) + beta*C as quadblas_qgemm_dev
 *                  (layout, transa, transb, m, n, k, A/lda, B/ldb, C/ldc);
 *   QBLAS_OP_GEMV: y = alpha*op(A)*x + beta*y as quadblas_qgemv_dev with
 *                  trans = transa, A/lda, x = B (incx = ldb), y = C (incy = ldc);
 *   QBLAS_OP_DOT : *C = sum_i x_i y_i with x = A (incx = lda), y = B
 *                  (incy = ldb), n elements.
 * All pointers are device pointers (16-byte aligned); alpha and beta hold
 * binary128 values (low word first).  quadblas_batch_plan cuts the problems
 * into equal-cost work items (granularity and gemm tile edge from the
 * autotuner) and uploads them; quadblas_batch_execute runs the whole batch on
 * `stream` with one memset and one persistent kernel and allocates nothing,
 * so it can be recorded in a CUDA graph and replayed; concurrent executions
 * of one plan must not overlap.  quadblas_batch_autotune times a calibration
 * batch at every pair of gemm tile edge (16, 32) and granularity (2^14 ..
 * 2^20 products per item) and caches the best pair per device (in memory and
 * in $QBLAS_AUTOTUNE_CACHE, default $HOME/.cache/qblas_gb300_autotune.txt).
 * Under quadblas_set_method(QBLAS_METHOD_OZAKI), qgemm problems with
 * m*n*k >= QBLAS_BATCH_OZAKI_MIN (environment, default 2^20) and k <= 8192
 * run, as their single calls would, on the tensor cores: all of them in one
 * grouped residue (CRT) chain of launches after the persistent kernel, in
 * the same stream; the plan then allocates their stacked operands and
 * residue planes (about 2 N (rows + 256-padded columns) k + 2 N 32768 x tiles
 * bytes for N moduli). */
enum { QBLAS_OP_GEMM = 0, QBLAS_OP_GEMV = 1, QBLAS_OP_DOT = 2 };

typedef struct {
  int32_t op;
  char layout, transa, transb, reserved;
  int64_t m, n, k;
  uint64_t alpha[2], beta[2];
  const void *A;
  int64_t lda;
  const void *B;
  int64_t ldb;
  void *C;
  int64_t ldc;
} qblas_problem;

int quadblas_batch_plan(const qblas_problem *problems, int64_t count, void **plan);
/* One batch, once (no plan kept): plan, execute on `stream`, wait for the
 * stream, free the plan.  For batches run more than once, keep a plan. */
int quadblas_qgemm_batched_dev(const qblas_problem *problems, int64_t count, void *stream);
int quadblas_batch_execute(void *plan, void *stream);
int quadblas_batch_destroy(void *plan);
/* info4: work items, granularity (products per item), blocks, split groups */
int quadblas_batch_info(void *plan, int64_t *info4);
/* info[0..n): work items, granularity, blocks, split groups, gemm tile edge,
 * qgemm problems on the grouped tensor-core path, their 128 x 256 tiles */
int quadblas_batch_info_ex(void *plan, int64_t *info, int64_t n);
int quadblas_batch_autotune(int64_t *grain_out);
/* The current device's setting for new plans (tuned, set, cached or default). */
int quadblas_batch_setting(int64_t *grain, int *tile);
/* Sets granularity (>= 256) and gemm tile edge (16 or 32; 0 keeps it). */
int quadblas_batch_configure(int64_t grain, int tile);
int quadblas_batch_set_grain(int64_t grain);
/* Smallest m*n*k routed to the grouped tensor-core path under the Ozaki
 * method, for plans built afterwards (0: QBLAS_BATCH_OZAKI_MIN or 2^20). */
int quadblas_batch_set_ozaki_min(int64_t products);
/* The same problems without the batch: one device-pointer call per problem
 * (quadblas_qgemm_dev with the soft-float method, or the Ozaki method for the
 * problems the batch gives to the tensor cores; quadblas_qgemv_dev,
 * quadblas_qdot_dev), in order, on `stream`, from a C loop.  It is the
 * one-call-per-problem baseline the batched launch is measured against, and
 * its results are bit-identical to quadblas_batch_execute's.  Returns the
 * first failing call's status. */
int quadblas_batch_run_serial(const qblas_problem *problems, int64_t count, void *stream);

/* ---- Configuration and errors (no reference counterpart) -------------- */
/* Method of qgemm and qgemv: QBLAS_METHOD_AUTO (soft-float for both),
 * _SOFTFLOAT or _OZAKI.  Ozaki qgemm is normwise accurate (set by the digit
 * count); Ozaki qgemv certifies every row's rounding and recomputes the rest
 * exactly, so its results equal the soft-float ones bit for bit. */
int quadblas_set_method(int method);
int quadblas_get_method(void);
/* Ozaki qgemm digit (slice) count per operand: 0 = default (16 of 9 bits, 18
 * of 8, 20 of 7), else 2..22; each call caps it by what the k dimension
 * allows (18 of 9 bits, 20 of 8, 22 of 7 at most).  qgemv uses its own fixed
 * split. */
int quadblas_set_ozaki_slices(int slices);
int quadblas_get_ozaki_slices(void);
/* Ozaki digit width: 0 = default (9), 7 or 8 bits per balanced digit (bf16
 * digit products) or 9 (fp16 digit products: fewer digit pairs for the same
 * bits, more k passes). */
int quadblas_set_ozaki_digit_bits(int bits);
int quadblas_get_ozaki_digit_bits(void);
/* Ozaki qgemm scheme: both truncate each operand to T = bits * slices - 1
 * bits after its row (column) scaling.  QBLAS_OZAKI_DIGITS multiplies every
 * digit pair whose weight the slice count keeps (slices (slices + 1) / 2
 * tensor-core products).  QBLAS_OZAKI_RESIDUES (Ozaki scheme II) multiplies
 * the operands' residues modulo N pairwise coprime moduli (N tensor-core
 * products, N about (2T + log2 k + 1) / 8.9) and recovers the exact integer
 * sum by the Chinese remainder theorem, so its only error is the
 * truncation.  QBLAS_OZAKI_AUTO (0, the default) takes residues whenever the
 * moduli table covers T and k (T <= 191 and at most 48 moduli), else
 * digits. */
enum { QBLAS_OZAKI_AUTO = 0, QBLAS_OZAKI_DIGITS = 1, QBLAS_OZAKI_RESIDUES = 2 };
int quadblas_set_ozaki_scheme(int scheme);
int quadblas_get_ozaki_scheme(void);
/* Phase timing of Ozaki qgemm calls (no reference counterpart): when
 * enabled, each call records CUDA events on its stream; read returns the
 * summed times in ms since the last read — out4[0] scaling and digit split,
 * out4[1] digit products on the tensor cores, out4[2] fold and epilogue —
 * and out4[3] the tensor flops of those calls (2*m*n*k*pairs).  on = 1
 * records every phase; on = 2 only the two events around the tensor-core
 * products (out4[0] and out4[2] stay 0), so that the kernels before and
 * after them, and consecutive calls, still overlap their launches. */
int quadblas_profile_enable(int on);
int quadblas_profile_read(double *out4, int *calls);
/* Frees the staging buffers that host-pointer calls keep on the current
 * device (they are allocated again, grown to need, by the next call), and
 * returns the unused memory of the library's scratch pool on that device
 * (device-pointer calls take their scratch from this pool in stream order
 * and give it back to the pool, which keeps it for the next call). */
int quadblas_release_buffers(void);
/* Testing aid for callers' failure handling: the next `count` device
 * allocations the library attempts fail as if the device were out of memory
 * (the call returns QBLAS_ERR_NO_MEMORY and leaves its outputs untouched);
 * 0 clears it.  Nothing is allocated for a failed attempt. */
int quadblas_debug_fail_allocations(int count);
/* Testing aid for callers' handling of device-side timeouts, without a
 * stalled GPU: the next Ozaki qgemm (which = 1; its tensor-core product
 * kernel) or Ozaki qgemv (which = 2) withholds one completion signal inside
 * its kernel and shortens that kernel's pipeline waits to 1 ms, so that a
 * wait runs out as it would on a real stall; the kernel then stops, waits
 * for its own copies and tensor-core operations in flight (1 s limit) and
 * frees its resources.  The qgemm then returns QBLAS_ERR_TIMEOUT (host
 * pointers) or sets the device flag read by quadblas_device_status, with NaN
 * in C; the qgemv recomputes every row exactly and returns correct results.
 * Calls after that one run normally. */
int quadblas_debug_stall_next_call(int which);
/* Testing aid for the certified rounding of qgemv: while on, every qgemv
 * records (in stream order) how many rows its exact pass recomputed because
 * their rounding could not be certified; quadblas_debug_exact_rows returns
 * the count of the last call once its stream has completed (-1 if never
 * enabled). */
int quadblas_debug_count_exact_rows(int on);
long long quadblas_debug_exact_rows(void);
/* Device-side failures of device-pointer calls (no reference counterpart).
 * The part 3 calls return before their kernels run, so a failure found on
 * the GPU cannot be their return value: an Ozaki qgemm whose tensor-core
 * kernels gave up on a wait (1 s without progress) leaves its C invalid (NaN
 * or unwritten) and sets a flag of the current device.  After synchronising the streams of the
 * calls in question, quadblas_device_status returns QBLAS_ERR_TIMEOUT if the
 * flag is set (QBLAS_OK otherwise) and clears it when `clear` is nonzero.
 * Host-pointer calls (parts 1 and 2) check their own call and return
 * QBLAS_ERR_TIMEOUT directly; they do not touch this flag.  (A qgemv whose
 * Ozaki kernel gives up still returns correct results: every row is then
 * recomputed exactly.) */
int quadblas_device_status(int clear);
/* Status of the calling thread's last call (part 1 calls record it too). */
int quadblas_last_error(void);
const char *quadblas_error_string(int code);

#ifdef __cplusplus
}
#endif

#endif /* QUADBLAS_GPU_H */
