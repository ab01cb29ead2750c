// Level-2 kernels: qgemv, y = alpha * op(A) x + beta * y.
//
// Replaces QuadBLAS::gemv_row_major / gemv_col_major
// (include/quadblas/algorithms/level2.hpp:15-100).  Each y_i is the
// correctly rounded exact sum_j op(A)(i,j) x_j (wide accumulator, one
// rounding) followed by the reference's epilogue
// y_i = fma(alpha, sum, beta * y_i) (level2.hpp:48; test_quadblas.cpp:172),
// so given the rounded sum the epilogue is bit-identical to the reference.
//
// Two memory layouts of op(A):
//  * rows contiguous (row-major, or column-major with trans): one warp per
//    row; lanes read consecutive 16-byte elements of the row (512 B per
//    warp per step) and x through the read-only cache.
//  * columns contiguous (column-major, or row-major with trans): one thread
//    per row, so a warp reads 32 consecutive elements of a column; the
//    columns are split into chunks over blockIdx.y to fill the GPU, each
//    (row, chunk) leaves a partial accumulator in scratch, and a second
//    kernel merges the chunks of each row in order and applies the epilogue.
#include "kernels.h"
#include "reduce.cuh"

namespace qb {

constexpr int kRowWarps = 8;  // warps per block of the row kernel

__device__ __forceinline__ q128 gemv_epilogue(q128 alpha, q128 sum, q128 beta, q128 yv) {
  return q_fma(alpha, sum, q_mul(beta, yv));
}

__global__ void __launch_bounds__(kRowWarps * 32)
    qgemv_rows_kernel(int64_t m, int64_t n, const q128* __restrict__ A, int64_t lda,
                      const q128* __restrict__ x, int64_t incx, q128 alpha, q128 beta,
                      q128* __restrict__ y, int64_t incy) {
  const int lane = threadIdx.x & 31;
  const int64_t warp0 = (int64_t)blockIdx.x * kRowWarps + (threadIdx.x >> 5);
  const int64_t nwarps = (int64_t)gridDim.x * kRowWarps;
  for (int64_t row = warp0; row < m; row += nwarps) {
    const q128* Ar = A + row * lda;
    wacc acc;
    wacc_init(acc);
    int64_t j = lane;
    for (; j + 96 < n; j += 128) {
      q128 a0 = ld_stream(Ar + j), a1 = ld_stream(Ar + j + 32);
      q128 a2 = ld_stream(Ar + j + 64), a3 = ld_stream(Ar + j + 96);
      q128 x0 = ld_cached(x + j * incx), x1 = ld_cached(x + (j + 32) * incx);
      q128 x2 = ld_cached(x + (j + 64) * incx), x3 = ld_cached(x + (j + 96) * incx);
      wacc_add_product(acc, qop_unpack(a0), qop_unpack(x0));
      wacc_add_product(acc, qop_unpack(a1), qop_unpack(x1));
      wacc_add_product(acc, qop_unpack(a2), qop_unpack(x2));
      wacc_add_product(acc, qop_unpack(a3), qop_unpack(x3));
    }
    for (; j < n; j += 32)
      wacc_add_product(acc, qop_unpack(ld_stream(Ar + j)), qop_unpack(ld_cached(x + j * incx)));
    wacc_warp_reduce(acc);
    if (lane == 0) {
      q128* yp = y + row * incy;
      *yp = gemv_epilogue(alpha, wacc_round(acc), beta, *yp);
    }
  }
}

constexpr int kColThreads = 128;

// Partial sums over columns [chunk*jc, min(n, (chunk+1)*jc)) for rows
// i = blockIdx.x*128 + threadIdx.x.  With nchunks == 1 the epilogue is
// applied directly; otherwise partials[chunk * m + i] is written.
__global__ void __launch_bounds__(kColThreads)
    qgemv_cols_kernel(int64_t m, int64_t n, const q128* __restrict__ A, int64_t lda,
                      const q128* __restrict__ x, int64_t incx, int64_t jc, q128 alpha, q128 beta,
                      q128* __restrict__ y, int64_t incy, wacc* __restrict__ partials) {
  const int64_t i = (int64_t)blockIdx.x * kColThreads + threadIdx.x;
  const int64_t chunk = blockIdx.y;
  int64_t j0 = chunk * jc, j1 = j0 + jc;
  if (j1 > n) j1 = n;
  if (i >= m) return;
  wacc acc;
  wacc_init(acc);
  int64_t j = j0;
  for (; j + 3 < j1; j += 4) {
    q128 a0 = ld_stream(A + j * lda + i), a1 = ld_stream(A + (j + 1) * lda + i);
    q128 a2 = ld_stream(A + (j + 2) * lda + i), a3 = ld_stream(A + (j + 3) * lda + i);
    q128 x0 = ld_cached(x + j * incx), x1 = ld_cached(x + (j + 1) * incx);
    q128 x2 = ld_cached(x + (j + 2) * incx), x3 = ld_cached(x + (j + 3) * incx);
    wacc_add_product(acc, qop_unpack(a0), qop_unpack(x0));
    wacc_add_product(acc, qop_unpack(a1), qop_unpack(x1));
    wacc_add_product(acc, qop_unpack(a2), qop_unpack(x2));
    wacc_add_product(acc, qop_unpack(a3), qop_unpack(x3));
  }
  for (; j < j1; ++j)
    wacc_add_product(acc, qop_unpack(ld_stream(A + j * lda + i)), qop_unpack(ld_cached(x + j * incx)));
  if (gridDim.y == 1) {
    q128* yp = y + i * incy;
    *yp = gemv_epilogue(alpha, wacc_round(acc), beta, *yp);
  } else {
    partials[chunk * m + i] = acc;
  }
}

__global__ void __launch_bounds__(kColThreads)
    qgemv_cols_finish_kernel(int64_t m, int64_t nchunks, const wacc* __restrict__ partials,
                             q128 alpha, q128 beta, q128* __restrict__ y, int64_t incy) {
  const int64_t i = (int64_t)blockIdx.x * kColThreads + threadIdx.x;
  if (i >= m) return;
  wacc acc;
  wacc_init(acc);
  for (int64_t c = 0; c < nchunks; ++c) wacc_merge(acc, partials[c * m + i]);
  q128* yp = y + i * incy;
  *yp = gemv_epilogue(alpha, wacc_round(acc), beta, *yp);
}

static int64_t col_chunks(int64_t m, int64_t n) {
  int64_t target_threads = (int64_t)device_sm_count() * 1536;
  int64_t c = (target_threads + m - 1) / (m > 0 ? m : 1);
  int64_t maxc = (n + 63) / 64;  // at least 64 columns per chunk
  if (c > maxc) c = maxc;
  if (c > 65535) c = 65535;
  if (c < 1) c = 1;
  return c;
}

size_t gemv_scratch_bytes(int64_t m, int64_t n, MatView A) {
  if (A.sj == 1 || m <= 0 || n <= 0) return 0;
  int64_t c = col_chunks(m, n);
  return c > 1 ? (size_t)c * (size_t)m * sizeof(wacc) : 0;
}

cudaError_t launch_gemv(int64_t m, int64_t n, q128 alpha, MatView A, const q128* x, int64_t incx,
                        q128 beta, q128* y, int64_t incy, void* scratch, cudaStream_t s) {
  if (m <= 0) return cudaSuccess;
  if (n <= 0) {
    // The reference returns without touching y when n == 0 (level2.hpp:21,61).
    return cudaSuccess;
  }
  if (A.sj == 1) {
    int64_t want = (m + kRowWarps - 1) / kRowWarps;
    int64_t cap = (int64_t)device_sm_count() * 8;
    int64_t nb = want < cap ? want : cap;
    qgemv_rows_kernel<<<(unsigned)nb, kRowWarps * 32, 0, s>>>(m, n, A.p, A.si, x, incx, alpha, beta,
                                                              y, incy);
    return cudaGetLastError();
  }
  int64_t c = col_chunks(m, n);
  int64_t jc = (n + c - 1) / c;
  c = (n + jc - 1) / jc;
  dim3 grid((unsigned)((m + kColThreads - 1) / kColThreads), (unsigned)c);
  wacc* partials = static_cast<wacc*>(scratch);
  qgemv_cols_kernel<<<grid, kColThreads, 0, s>>>(m, n, A.p, A.sj, x, incx, jc, alpha, beta, y, incy,
                                                 partials);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || c == 1) return e;
  qgemv_cols_finish_kernel<<<(unsigned)((m + kColThreads - 1) / kColThreads), kColThreads, 0, s>>>(
      m, c, partials, alpha, beta, y, incy);
  return cudaGetLastError();
}

}  // namespace qb
