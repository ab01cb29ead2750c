// Level-2 kernels: qgemv, y = alpha * op(A) x + beta * y.
//
// Replaces QuadBLAS::gemv_row_major / gemv_col_major
// (include/quadblas/algorithms/level2.hpp:15-100).  Each y_i is the
// correctly rounded exact sum_j op(A)(i,j) x_j (wide accumulator, one
// rounding) followed by the reference's epilogue
// y_i = fma(alpha, sum, beta * y_i) (level2.hpp:48; test_quadblas.cpp:172),
// so given the rounded sum the epilogue is bit-identical to the reference.
//
// x is unpacked once per call into scratch (significand at bit 127,
// exponent, sign and class), since every element of x is used m times.
// Two memory layouts of op(A):
//  * rows contiguous (row-major, or column-major with trans) and m < 4096:
//    a row is shared by 1, 2, 4 or 8 warps of a 256-thread block (more warps for
//    longer rows); lanes read consecutive 16-byte elements (512 B per warp
//    per step) and the warps' accumulators are merged in shared memory in a
//    fixed order.  One block per 8/wpr rows keeps the grid fine-grained.
//  * one thread per row (columns contiguous, i.e. column-major or row-major
//    with trans, where a warp reads 32 consecutive elements of a column; and
//    rows contiguous with m >= 4096, where each lane reads its row through
//    L1): all lanes share each x_j; the columns are split into chunks over
//    blockIdx.y to fill the GPU, each (row, chunk) leaves a partial
//    accumulator in scratch, and a second kernel merges the chunks of each
//    row in order and applies the epilogue.
#include <stddef.h>

#include "exact.cuh"
#include "gemv_rows.cuh"
#include "kernels.h"
#include "reduce.cuh"

namespace qb {

__device__ __forceinline__ q128 gemv_epilogue(q128 alpha, q128 sum, q128 beta, q128 yv) {
  return q_epilogue(alpha, sum, beta, yv);
}

// ---- x unpacked once -------------------------------------------------------
__global__ void qop_unpack_kernel(int64_t n, const q128* __restrict__ x, int64_t incx,
                                  uint4* __restrict__ xm, int2* __restrict__ xe, RowList* __restrict__ L) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  if (blockIdx.x == 0 && threadIdx.x == 0) L->count = 0;  // this call's list starts empty
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    qop o = qop_unpack(ld_cached(x + i * incx));
    xm[i] = make_uint4(o.m0, o.m1, o.m2, o.m3);
    xe[i] = make_int2(o.e, (int)(o.s | (o.cls << 1)));
  }
}

__device__ __forceinline__ qop qop_fetch(const uint4* __restrict__ xm, const int2* __restrict__ xe,
                                         int64_t i) {
  uint4 m = __ldg(xm + i);
  int2 e = __ldg(xe + i);
  qop o;
  o.m0 = m.x;
  o.m1 = m.y;
  o.m2 = m.z;
  o.m3 = m.w;
  o.e = e.x;
  o.s = (uint32_t)e.y & 1u;
  o.cls = (uint32_t)e.y >> 1;
  return o;
}

// ---- rows contiguous ------------------------------------------------------
constexpr int kRowThreads = 256;

__global__ void __launch_bounds__(kRowThreads, 4)
    qgemv_rows_kernel(int64_t m, int64_t n, const q128* __restrict__ A, int64_t lda,
                      const uint4* __restrict__ xm, const int2* __restrict__ xe, int wpr_log2,
                      q128 alpha, q128 beta, q128* __restrict__ y, int64_t incy, RowList* __restrict__ L) {
  __shared__ wacc sm[kRowThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wpr = 1 << wpr_log2;
  const int sub = warp & (wpr - 1);
  const int64_t row = (int64_t)blockIdx.x * ((kRowThreads / 32) >> wpr_log2) + (warp >> wpr_log2);
  wacc acc;
  wacc_init(acc);
  if (row < m) {
    const q128* Ar = A + row * lda;
    const int64_t step = 32 * (int64_t)wpr;
    int64_t j = (int64_t)sub * 32 + lane;
    for (; j + 3 * step < n; j += 4 * step) {
      q128 a0 = ld_stream(Ar + j), a1 = ld_stream(Ar + j + step);
      q128 a2 = ld_stream(Ar + j + 2 * step), a3 = ld_stream(Ar + j + 3 * step);
      wacc_add_product(acc, qop_unpack(a0), qop_fetch(xm, xe, j));
      wacc_add_product(acc, qop_unpack(a1), qop_fetch(xm, xe, j + step));
      wacc_add_product(acc, qop_unpack(a2), qop_fetch(xm, xe, j + 2 * step));
      wacc_add_product(acc, qop_unpack(a3), qop_fetch(xm, xe, j + 3 * step));
    }
    for (; j < n; j += step) wacc_add_product(acc, qop_unpack(ld_stream(Ar + j)), qop_fetch(xm, xe, j));
  }
  wacc_warp_reduce(acc);
  if (lane == 0) sm[warp] = acc;
  __syncthreads();
  if (lane == 0 && sub == 0 && row < m) {
    wacc a = sm[warp];
    for (int k = 1; k < wpr; ++k) wacc_merge(a, sm[warp + k]);
    // budget: 2 per product, 3 per merge (31 per warp and wpr - 1 between warps)
    const uint64_t err = 2 * (uint64_t)n + 3 * (32 * (uint64_t)wpr + 8);
    gemv_finish_row(alpha, a, err, beta, y + row * incy, row, L);
  }
}

// ---- one thread per row --------------------------------------------------
constexpr int kColThreads = 128;

// Partial sums over columns [chunk*jc, min(n, (chunk+1)*jc)) for rows
// i = blockIdx.x*128 + threadIdx.x: all lanes of a warp read the same x_j
// (a broadcast) and keep one accumulator each, with no reduction across
// lanes.  kRowMajor: op(A)(i, j) = A[i*ld + j], each lane reads its own row
// through L1 (one 128-byte line serves eight consecutive columns);
// otherwise A[j*ld + i], where a warp's loads are coalesced and read once.
// With one chunk the epilogue is applied directly; otherwise
// partials[chunk * m + i] is written.
template <bool kRowMajor>
__global__ void __launch_bounds__(kColThreads)
    qgemv_lane_kernel(int64_t m, int64_t n, const q128* __restrict__ A, int64_t ld,
                      const uint4* __restrict__ xm, const int2* __restrict__ xe, int64_t jc,
                      q128 alpha, q128 beta, q128* __restrict__ y, int64_t incy,
                      wacc* __restrict__ partials, RowList* __restrict__ L) {
  const int64_t i = (int64_t)blockIdx.x * kColThreads + threadIdx.x;
  const int64_t chunk = blockIdx.y;
  int64_t j0 = chunk * jc, j1 = j0 + jc;
  if (j1 > n) j1 = n;
  if (i >= m) return;
  auto ldA = [&](int64_t j) { return kRowMajor ? ld_cached(A + i * ld + j) : ld_stream(A + j * ld + i); };
  wacc acc;
  wacc_init(acc);
  int64_t j = j0;
  for (; j + 3 < j1; j += 4) {
    q128 a0 = ldA(j), a1 = ldA(j + 1), a2 = ldA(j + 2), a3 = ldA(j + 3);
    wacc_add_product(acc, qop_unpack(a0), qop_fetch(xm, xe, j));
    wacc_add_product(acc, qop_unpack(a1), qop_fetch(xm, xe, j + 1));
    wacc_add_product(acc, qop_unpack(a2), qop_fetch(xm, xe, j + 2));
    wacc_add_product(acc, qop_unpack(a3), qop_fetch(xm, xe, j + 3));
  }
  for (; j < j1; ++j) wacc_add_product(acc, qop_unpack(ldA(j)), qop_fetch(xm, xe, j));
  if (gridDim.y == 1)
    gemv_finish_row(alpha, acc, 2 * (uint64_t)n + 3, beta, y + i * incy, i, L);
  else
    partials[chunk * m + i] = acc;
}

__global__ void __launch_bounds__(kColThreads)
    qgemv_cols_finish_kernel(int64_t m, int64_t n, int64_t nchunks, const wacc* __restrict__ partials,
                             q128 alpha, q128 beta, q128* __restrict__ y, int64_t incy,
                             RowList* __restrict__ L) {
  const int64_t i = (int64_t)blockIdx.x * kColThreads + threadIdx.x;
  if (i >= m) return;
  wacc acc;
  wacc_init(acc);
  for (int64_t c = 0; c < nchunks; ++c) wacc_merge(acc, partials[c * m + i]);
  gemv_finish_row(alpha, acc, 2 * (uint64_t)n + 3 * ((uint64_t)nchunks + 2), beta, y + i * incy, i, L);
}

// Recomputation of the listed rows, one block per row.  With try_wide the
// block first sums the row in wide accumulators (one per thread, merged in
// shared memory) and certifies that rounding, which settles the rows whose
// Ozaki bound was too loose; the rest (and every row when !try_wide: the
// soft-float kernels already tried the wide accumulator) are summed exactly
// by a Kulisch accumulator.
constexpr int kExactThreads = 512;

__global__ void __launch_bounds__(kExactThreads)
    qgemv_exact_kernel(const RowList* __restrict__ L, int64_t n, MatView A, const q128* __restrict__ x,
                       int64_t incx, q128 alpha, q128 beta, q128* __restrict__ y, int64_t incy, int try_wide) {
  __shared__ KulischBlock K;
  __shared__ wacc sm[kExactThreads / 32];
  __shared__ int done;
  const unsigned cnt = *reinterpret_cast<const volatile unsigned*>(&L->count);
  for (unsigned t = blockIdx.x; t < cnt; t += gridDim.x) {
    const int64_t i = L->row[t];
    q128* yp = y + i * incy;
    if (try_wide) {
      wacc acc;
      wacc_init(acc);
      const q128* Ar = A.p + i * A.si;
      const int64_t step = blockDim.x;
      int64_t j = threadIdx.x;
      for (; j + 3 * step < n; j += 4 * step) {  // four element pairs in flight
        q128 a0 = ld_cached(Ar + j * A.sj), a1 = ld_cached(Ar + (j + step) * A.sj);
        q128 a2 = ld_cached(Ar + (j + 2 * step) * A.sj), a3 = ld_cached(Ar + (j + 3 * step) * A.sj);
        q128 x0 = ld_cached(x + j * incx), x1 = ld_cached(x + (j + step) * incx);
        q128 x2 = ld_cached(x + (j + 2 * step) * incx), x3 = ld_cached(x + (j + 3 * step) * incx);
        wacc_add_product(acc, qop_unpack(a0), qop_unpack(x0));
        wacc_add_product(acc, qop_unpack(a1), qop_unpack(x1));
        wacc_add_product(acc, qop_unpack(a2), qop_unpack(x2));
        wacc_add_product(acc, qop_unpack(a3), qop_unpack(x3));
      }
      for (; j < n; j += step) wacc_add_product(acc, qop_unpack(ld_cached(Ar + j * A.sj)), qop_unpack(ld_cached(x + j * incx)));
      wacc_block_reduce(acc, sm);
      if (threadIdx.x == 0) {
        q128 r;
        done = wacc_round_certified(acc, 2 * (uint64_t)n + 3 * kExactThreads, r);
        if (done) *yp = q_epilogue(alpha, r, beta, *yp);
      }
      __syncthreads();
      if (done) continue;
    }
    q128 r = block_exact_dot(K, n, A.p + i * A.si, A.sj, x, incx);
    if (threadIdx.x == 0) *yp = q_epilogue(alpha, r, beta, *yp);
  }
}

// Row-major op(A) with at least this many rows uses the thread-per-row
// kernel (measured at 8192 x 8192: 2370 GB/s against 2170 for warps per
// row; with few long rows the column chunks' merges cost more than they save).
constexpr int64_t kLaneRowsMin = 4096;

static bool use_lanes(int64_t m, const MatView& A) { return A.sj != 1 || m >= kLaneRowsMin; }

// Column chunks of the thread-per-row kernel: enough (row, chunk) threads
// to fill the GPU (two per resident thread slot for long row-major runs),
// at least 64 columns each.
static int64_t col_chunks(int64_t m, int64_t n, bool row_major) {
  int64_t target_threads = (int64_t)device_sm_count() * (row_major && m >= 8192 ? 3072 : 1536);
  int64_t c = (target_threads + m - 1) / (m > 0 ? m : 1);
  int64_t maxc = (n + 63) / 64;
  if (c > maxc) c = maxc;
  if (c > 65535) c = 65535;
  if (c < 1) c = 1;
  return c;
}

static unsigned* g_exact_rows = nullptr;
void gemv_count_exact_rows(unsigned* host_pinned) { g_exact_rows = host_pinned; }

// Exact pass over the listed rows (returns at once when none), then the
// optional record of how many there were.
static cudaError_t launch_exact_rows(RowList* L, int64_t n, MatView A, const q128* x, int64_t incx, q128 alpha,
                                     q128 beta, q128* y, int64_t incy, cudaStream_t s, bool try_wide) {
  qgemv_exact_kernel<<<(unsigned)device_sm_count(), kExactThreads, 0, s>>>(L, n, A, x, incx, alpha, beta, y,
                                                                           incy, try_wide ? 1 : 0);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && g_exact_rows)
    e = cudaMemcpyAsync(g_exact_rows, &L->count, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  return e;
}

static size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

static size_t rowlist_bytes(int64_t m) { return round256(offsetof(RowList, row) + (size_t)m * 8); }

// The Ozaki kernels run when asked for (method 2); the library's own choice
// stays with the soft-float kernels, which are faster at every size measured.
static bool use_ozaki(int64_t m, int64_t n, int method) {
  (void)m;
  (void)n;
  return method == 2;
}

// Scratch: [uncertified rows][Ozaki buffers], or
// [x significands: 16n][x exponents: 8n][uncertified rows] (+ column partials)
size_t gemv_scratch_bytes(int64_t m, int64_t n, MatView A, int method) {
  if (m <= 0 || n <= 0) return 0;
  if (use_ozaki(m, n, method)) return rowlist_bytes(m) + gemv_ozaki_scratch_bytes(m, n);
  size_t xs = round256((size_t)n * 16) + round256((size_t)n * 8) + rowlist_bytes(m);
  if (!use_lanes(m, A)) return xs;
  int64_t c = col_chunks(m, n, A.sj == 1);
  return xs + (c > 1 ? (size_t)c * (size_t)m * sizeof(wacc) : 0);
}

// Warps per row: enough lanes that each has at least 64 terms.
static int rows_wpr_log2(int64_t n) {
  int l = 0;
  while (l < 3 && n >= (int64_t)(32 << (l + 1)) * 64) ++l;
  return l;
}

cudaError_t launch_gemv(int64_t m, int64_t n, q128 alpha, MatView A, const q128* x, int64_t incx,
                        q128 beta, q128* y, int64_t incy, void* scratch, cudaStream_t s, int method) {
  if (m <= 0) return cudaSuccess;
  if (n <= 0) return cudaSuccess;  // the reference leaves y untouched (level2.hpp:21,61)
  char* base = static_cast<char*>(scratch);
  if (use_ozaki(m, n, method)) {
    RowList* L = reinterpret_cast<RowList*>(base);
    cudaError_t e = launch_gemv_ozaki(m, n, alpha, A, x, incx, beta, y, incy, L, base + rowlist_bytes(m), s);
    if (e != cudaSuccess) return e;
    return launch_exact_rows(L, n, A, x, incx, alpha, beta, y, incy, s, true);
  }
  uint4* xm = reinterpret_cast<uint4*>(base);
  int2* xe = reinterpret_cast<int2*>(base + round256((size_t)n * 16));
  RowList* L = reinterpret_cast<RowList*>(base + round256((size_t)n * 16) + round256((size_t)n * 8));
  {
    int64_t nb = (n + 255) / 256;
    int64_t cap = (int64_t)device_sm_count() * 4;
    qop_unpack_kernel<<<(unsigned)(nb < cap ? nb : cap), 256, 0, s>>>(n, x, incx, xm, xe, L);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  cudaError_t e;
  if (!use_lanes(m, A)) {
    int l = rows_wpr_log2(n);
    int64_t rows_per_block = (kRowThreads / 32) >> l;
    int64_t nb = (m + rows_per_block - 1) / rows_per_block;
    if (nb > 0x7fffffff) return cudaErrorInvalidConfiguration;
    qgemv_rows_kernel<<<(unsigned)nb, kRowThreads, 0, s>>>(m, n, A.p, A.si, xm, xe, l, alpha, beta,
                                                           y, incy, L);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  } else {
    const bool row_major = A.sj == 1;
    int64_t c = col_chunks(m, n, row_major);
    int64_t jc = (n + c - 1) / c;
    c = (n + jc - 1) / jc;
    dim3 grid((unsigned)((m + kColThreads - 1) / kColThreads), (unsigned)c);
    size_t xs = round256((size_t)n * 16) + round256((size_t)n * 8) + rowlist_bytes(m);
    wacc* partials = reinterpret_cast<wacc*>(base + xs);
    if (row_major)
      qgemv_lane_kernel<true><<<grid, kColThreads, 0, s>>>(m, n, A.p, A.si, xm, xe, jc, alpha, beta, y, incy,
                                                           partials, L);
    else
      qgemv_lane_kernel<false><<<grid, kColThreads, 0, s>>>(m, n, A.p, A.sj, xm, xe, jc, alpha, beta, y,
                                                            incy, partials, L);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (c > 1) {
      qgemv_cols_finish_kernel<<<(unsigned)((m + kColThreads - 1) / kColThreads), kColThreads, 0, s>>>(
          m, n, c, partials, alpha, beta, y, incy, L);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
  }
  return launch_exact_rows(L, n, A, x, incx, alpha, beta, y, incy, s, false);
}

}  // namespace qb
