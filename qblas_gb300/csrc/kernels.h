// Internal interface between the C ABI layer (capi.cpp) and the CUDA
// kernels.  All pointers are device pointers; all strides are in elements
// (16-byte binary128 values) and positive.  Every launcher is stream-ordered
// and allocates nothing: scratch memory, when a kernel needs it, is passed
// in by the caller and its size is given by the matching *_scratch_bytes().
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "softquad.cuh"

namespace qb {

// Error codes of the C ABI (mirrored in include/quadblas_gpu.h).
enum Status : int {
  kOk = 0,
  kErrInvalidValue = 1,
  kErrCuda = 2,
  kErrNoMemory = 3,
  kErrNotSupported = 4,
  kErrNoDevice = 5,
  kErrMisaligned = 6,
  kErrTimeout = 7,
};

// op(A) is an m x n matrix with element (i, j) at A[i*si + j*sj].
struct MatView {
  const q128* p;
  int64_t si, sj;
};

// ---- level 1 -----------------------------------------------------------
// out[0] = round(sum_i x_i*y_i)  (sqrt of it when take_sqrt != 0)
size_t dot_scratch_bytes(int64_t n);
cudaError_t launch_dot(int64_t n, const q128* x, int64_t incx, const q128* y, int64_t incy,
                       q128* out, int take_sqrt, void* scratch, cudaStream_t s);
// y_i = fma(alpha, x_i, y_i)
cudaError_t launch_axpy(int64_t n, q128 alpha, const q128* x, int64_t incx, q128* y, int64_t incy,
                        cudaStream_t s);

// ---- level 2 -----------------------------------------------------------
// y_i = fma(alpha, round(sum_j op(A)(i,j) x_j), beta * y_i), i < m.
// method: 0 chooses (Ozaki split on the tensor cores for large matrices,
// soft-float otherwise), 1 soft-float, 2 Ozaki; the results are identical.
size_t gemv_scratch_bytes(int64_t m, int64_t n, MatView A, int method);
// When set (pinned host memory), every qgemv call copies the number of rows
// its exact pass recomputed there, in stream order; nullptr stops it.
void gemv_count_exact_rows(unsigned* host_pinned);
cudaError_t launch_gemv(int64_t m, int64_t n, q128 alpha, MatView A, const q128* x, int64_t incx,
                        q128 beta, q128* y, int64_t incy, void* scratch, cudaStream_t s, int method);

// ---- level 3 -----------------------------------------------------------
struct GemmArgs {
  int64_t m, n, k;
  const q128* A;
  int64_t sai, sal;  // op(A)(i, l) = A[i*sai + l*sal]
  const q128* B;
  int64_t sbl, sbj;  // op(B)(l, j) = B[l*sbl + j*sbj]
  q128* C;
  int64_t sci, scj;  // C(i, j) = C[i*sci + j*scj]
  q128 alpha, beta;
};
// C = fma(alpha, round(sum_l op(A)(i,l) op(B)(l,j)), beta * C), soft-float
cudaError_t launch_gemm_softfloat(const GemmArgs& g, cudaStream_t s);

// C = fma(alpha, round(sum), beta * C) with the sum from an Ozaki split on
// the tensor cores, both schemes truncating the operands to T = bits *
// digits - 1 bits: `scheme` 1 = balanced digits of `bits` = 7, 8 or 9 bits
// and their digit-pair products (ozaki.cuh); 0 or 2 = residues modulo
// pairwise coprime moduli and the Chinese remainder theorem (ozcrt.cuh)
// whenever its table fits T and k, else digit pairs.
int ozaki_default_digit_bits();
int ozaki_default_digits(int bits);
// Largest digit count whose 192-bit fold cannot overflow for inner dimension k.
int ozaki_digit_cap(int bits, int64_t k);
size_t ozaki_scratch_bytes(int64_t m, int64_t n, int64_t k, int digits, int bits, int scheme);
size_t ozaki_error_flag_offset(int64_t m, int64_t n, int64_t k, int digits, int bits, int scheme);
bool ozaki_uses_crt(int64_t k, int digits, int bits, int scheme);
// Optional overlap for callers that copy op(B) and C to the device
// themselves: the op(B) side (its scales and digits) runs on `b_stream`,
// in stream order after the copy of B that the caller put there, while op(A)
// is cut on the main stream; the digit products wait for the op(B) side
// (`b_done`, recorded here) and the fold waits for `c_ready` (the caller's
// copy of C).
// When `band_done` is set and C's rows are contiguous, the fold runs in row
// bands and band_done(band_ctx, i0, i1) is called after each band's fold is
// enqueued (rows [i0, i1) of C are then final in stream order), so that the
// caller can copy a band out while the next one is folded.
//
// When `a_rows` is set, op(A) is cut into digits band by band on `a_stream`:
// a_rows(a_ctx, r0, r1, a_stream) is called before each band and must make
// a_stream wait until rows [r0, r1) of op(A) are on the device (so that the
// caller can copy A in row bands); the digit products of the tiles that
// need a band start as soon as it is cut (`a_done` is recorded for that).
struct OzakiOverlap {
  cudaStream_t b_stream;
  cudaEvent_t b_done;
  cudaEvent_t c_ready;
  int (*band_done)(void* ctx, int64_t i0, int64_t i1);
  void* band_ctx;
  int (*a_rows)(void* ctx, int64_t r0, int64_t r1, cudaStream_t s);
  void* a_ctx;
  cudaStream_t a_stream;
  cudaEvent_t a_done;
  // nonzero: a_rows also copies the same rows of C and records c_ready after
  // them, so rows of C can be folded as soon as their products are done
  int c_banded;
};
// `report`, when not null, is a device-accessible word (mapped host memory)
// that the fold sets to 1 if a wait of the tensor-core kernel timed out.
cudaError_t launch_gemm_ozaki(const GemmArgs& g, int digits, int bits, void* scratch,
                              cudaStream_t s, const OzakiOverlap* overlap = nullptr, int scheme = 0,
                              int* report = nullptr);
// Grouped residue (CRT) qgemm: many problems through one chain of launches
// (gather, scales, residues, products, reconstruction), bit-identical to
// launch_gemm_ozaki of each problem with the same digits, bits and scheme.
// op(A) rows of every problem are stacked (each problem padded to 128 rows)
// into a_all, op(B)'s columns into b_all (256-row padding) as rows of
// k_pad elements; the products run over a list of (128-row A tile, 256-row
// B tile) pairs whose reduced residues are stored tile-major, and the
// reconstruction writes each tile's outputs through its problem's C.
struct OzakiGroupRow {      // one stacked row: len elements from p, stride apart
  const q128* p;
  int64_t stride, len;
};
struct OzakiGroupTile {     // a_tile: 128-row tile of a_all; b_tile: 256-row tile of b_all
  int32_t a_tile, b_tile, prob, row0, col0, pad[3];
};
struct OzakiGroupProb {
  q128* C;
  int64_t sci, scj, m, n, k;
  q128 alpha, beta;
  const q128* A;
  int64_t sai, sal;
  const q128* B;
  int64_t sbl, sbj;
};
struct OzakiGroup {
  int64_t rows_a, rows_b, k_pad, ntiles;  // rows_a % 128 == 0, rows_b % 256 == 0, k_pad % 64 == 0
  int64_t k_max;                          // largest k (sets the moduli)
  int digits, bits;
  const OzakiGroupRow* rows;              // rows_a + rows_b (device)
  const OzakiGroupTile* tiles;            // ntiles (device)
  const OzakiGroupProb* probs;            // (device)
  q128* a_all;                            // rows_a x k_pad, zero where no row element is gathered
  q128* b_all;                            // rows_b x k_pad, likewise
  void* scratch;                          // ozaki_group_scratch_bytes
};
// 0 when the residue scheme has no table for these digits, bits and k.
size_t ozaki_group_scratch_bytes(int64_t rows_a, int64_t rows_b, int64_t k_pad, int64_t ntiles, int64_t k_max,
                                 int digits, int bits);
cudaError_t launch_gemm_ozaki_grouped(const OzakiGroup& G, cudaStream_t s);
// The library's current qgemm settings (quadblas_set_method, _ozaki_slices,
// _ozaki_digit_bits, _ozaki_scheme and their environment defaults): method
// (1 soft-float, 2 Ozaki), digits for inner dimension k, bits, scheme.
int gemm_method_setting();
int gemm_digits_setting(int64_t k);
int gemm_bits_setting();
int ozaki_scheme_setting();
// Whether a batched qgemm problem of this shape runs on the grouped residue
// path under the current settings (and the one-by-one baseline then makes
// the Ozaki call for it): method 2, residue scheme available for k <= 8192
// with the same digits as at k = 8192, and m n k at least the threshold
// (QBLAS_BATCH_OZAKI_MIN, default 2^20 products).
bool batch_gemm_routed(int64_t m, int64_t n, int64_t k);

// Test hooks: the next Ozaki qgemm product launch / Ozaki qgemv launch
// withholds one accumulator-full commit with 1 ms pipeline waits.
void ozaki_debug_stall_next();
void ozgemv_debug_stall_next();
// Phase timing of Ozaki calls with CUDA events (off by default).
void ozaki_profile_enable(int mode);  // 0 off, 1 every phase, 2 the products only
int ozaki_profile_read(double* out4, int* calls);

// Multiprocessor count of the current device (cached).
// Every device allocation of the library goes through these: they fail
// with cudaErrorMemoryAllocation, allocating nothing, while an injected
// failure count (quadblas_debug_fail_allocations) is pending.
cudaError_t dev_malloc(void** p, size_t bytes);
cudaError_t dev_malloc_async(void** p, size_t bytes, cudaStream_t s);
// The library's stream-ordered scratch pool of device `dev` (keeps freed
// memory until quadblas_release_buffers), or null.
cudaMemPool_t scratch_pool(int dev);
int device_sm_count();

// Blocks of `kernel` (with `threads` threads and `smem` dynamic shared
// memory) that fit on one multiprocessor of the current device.
int resident_blocks_per_sm(const void* kernel, int threads, size_t smem);

}  // namespace qb
