// Level-1 kernels: qdot / qnrm2 and qaxpy.
//
// qdot replaces QuadBLAS::dot (include/quadblas/algorithms/level1.hpp:80-137)
// and qaxpy replaces QuadBLAS::axpy (level1.hpp:190-223).
//
// qdot is HBM-bound: each term reads two 16-byte elements.  A grid of
// (SM count x resident blocks) threads streams the vectors with coalesced
// 16-byte loads, every thread keeps one wide accumulator (wacc.cuh), the
// block merges its threads' accumulators (warp shuffles + shared memory),
// and a second single-block kernel merges the per-block partials in a
// fixed order and rounds once.  The products skip the partial products that
// only feed their lowest 64 bits (three multiplies of 31, on the saturated
// fmaheavy pipe), which adds less than 2^34 units of the frame's last bit per
// term to the error budget.  The rounding is certified against that budget
// (exact.cuh); if the sum cancels below it, a third kernel recomputes the
// sum exactly (Kulisch accumulator) — it returns at once otherwise.
#include <atomic>

#include "exact.cuh"
#include "kernels.h"
#include "reduce.cuh"

namespace qb {

constexpr int kDotThreads = 256;
constexpr int kDotBlocksPerSm = 4;

// Per-device caches below are atomics: host threads may call on one device
// at the same time; they compute the same value, so the last store wins.
int device_sm_count() {
  static std::atomic<int> cached[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
  int v = cached[dev].load(std::memory_order_relaxed);
  if (!v) {
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
      v = 148;
    cached[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

int resident_blocks_per_sm(const void* kernel, int threads, size_t smem) {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, threads, smem) != cudaSuccess ||
      nb < 1) {
    cudaGetLastError();
    nb = 1;
  }
  return nb;
}



__global__ void __launch_bounds__(kDotThreads, 4)
    qdot_partial_kernel(int64_t n, const q128* __restrict__ x, int64_t incx,
                        const q128* __restrict__ y, int64_t incy, wacc* __restrict__ partials) {
  __shared__ wacc sm[kDotThreads / 32];
  wacc acc;
  wacc_init(acc);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (incx == 1 && incy == 1) {
    for (; i + 3 * stride < n; i += 4 * stride) {
      q128 xa = ld_stream(x + i), ya = ld_stream(y + i);
      q128 xb = ld_stream(x + i + stride), yb = ld_stream(y + i + stride);
      q128 xc = ld_stream(x + i + 2 * stride), yc = ld_stream(y + i + 2 * stride);
      q128 xd = ld_stream(x + i + 3 * stride), yd = ld_stream(y + i + 3 * stride);
      wacc_add_product_trunc(acc, qop_unpack(xa), qop_unpack(ya));
      wacc_add_product_trunc(acc, qop_unpack(xb), qop_unpack(yb));
      wacc_add_product_trunc(acc, qop_unpack(xc), qop_unpack(yc));
      wacc_add_product_trunc(acc, qop_unpack(xd), qop_unpack(yd));
    }
  }
  for (; i < n; i += stride)
    wacc_add_product_trunc(acc, qop_unpack(ld_stream(x + i * incx)), qop_unpack(ld_stream(y + i * incy)));
  wacc_block_reduce(acc, sm);
  if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

// Merges `count` partials; writes the rounded value (or its square root)
// when the rounding is certified for the error budget `err`, otherwise
// arms and resets the exact pass in G.
__global__ void __launch_bounds__(kDotThreads)
    wacc_finalize_kernel(const wacc* __restrict__ partials, int64_t count, q128* __restrict__ out,
                         int take_sqrt, uint64_t err, ExactGlobal* __restrict__ G) {
  __shared__ wacc sm[kDotThreads / 32];
  __shared__ int need;
  wacc acc;
  wacc_init(acc);
  for (int64_t j = threadIdx.x; j < count; j += blockDim.x) wacc_merge(acc, partials[j]);
  wacc_block_reduce(acc, sm);
  if (threadIdx.x == 0) {
    q128 r;
    const bool ok = wacc_round_certified(acc, err, r);
    if (ok) *out = take_sqrt ? q_sqrt(r) : r;
    need = ok ? 0 : 1;
    G->need = need;
  }
  __syncthreads();
  if (need) exact_global_reset(G);
}

// The exact pass: every block adds its share of the products to a
// Kulisch accumulator; the last block rounds (and takes the square root).
__global__ void __launch_bounds__(kDotThreads)
    qdot_exact_kernel(int64_t n, const q128* __restrict__ x, int64_t incx, const q128* __restrict__ y,
                      int64_t incy, ExactGlobal* __restrict__ G, q128* __restrict__ out, int take_sqrt) {
  __shared__ KulischBlock K;
  if (!*reinterpret_cast<volatile int*>(&G->need)) return;
  q128 r;
  if (grid_exact_dot(K, G, n, x, incx, y, incy, &r) && threadIdx.x == 0) *out = take_sqrt ? q_sqrt(r) : r;
}

// One wave of resident blocks (no tail wave), fewer for short vectors.
static int64_t dot_blocks(int64_t n) {
  static std::atomic<int> cached[64];
  int dev = 0;
  cudaGetDevice(&dev);
  int per_sm = kDotBlocksPerSm;
  if (dev >= 0 && dev < 64) {
    int c = cached[dev].load(std::memory_order_relaxed);
    if (!c) {
      c = resident_blocks_per_sm((const void*)qdot_partial_kernel, kDotThreads, 0);
      cached[dev].store(c, std::memory_order_relaxed);
    }
    per_sm = c < kDotBlocksPerSm ? c : kDotBlocksPerSm;
  }
  int64_t per_block = (int64_t)kDotThreads * 4;  // at least 4 terms per thread
  int64_t want = (n + per_block - 1) / per_block;
  int64_t cap = (int64_t)device_sm_count() * per_sm;
  if (want < 1) want = 1;
  return want < cap ? want : cap;
}

static size_t dot_partials_bytes(int64_t n) {
  return ((size_t)dot_blocks(n) * sizeof(wacc) + 255) / 256 * 256;
}

// Block partials, then the exact pass's state.
size_t dot_scratch_bytes(int64_t n) { return dot_partials_bytes(n) + sizeof(ExactGlobal); }

__global__ void qzero_kernel(q128* out, int take_sqrt) {
  (void)take_sqrt;
  *out = q_zero(0);
}

cudaError_t launch_dot(int64_t n, const q128* x, int64_t incx, const q128* y, int64_t incy,
                       q128* out, int take_sqrt, void* scratch, cudaStream_t s) {
  if (n <= 0) {
    qzero_kernel<<<1, 1, 0, s>>>(out, take_sqrt);
    return cudaGetLastError();
  }
  int64_t nb = dot_blocks(n);
  wacc* partials = static_cast<wacc*>(scratch);
  ExactGlobal* G = reinterpret_cast<ExactGlobal*>(static_cast<char*>(scratch) + dot_partials_bytes(n));
  qdot_partial_kernel<<<(unsigned)nb, kDotThreads, 0, s>>>(n, x, incx, y, incy, partials);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // truncation budget: 2 units per product, 3 per merge (every thread's
  // accumulator, the block partials and the final block's merges)
  // budget: 2^34 + 2 units per (truncated) product, 3 per merge; beyond
  // 2^29 terms it saturates and the exact pass decides
  const uint64_t merges = 3 * ((uint64_t)nb * kDotThreads + (uint64_t)nb + 2 * kDotThreads + 64);
  const uint64_t err = n > ((int64_t)1 << 29) ? ~0ull : (uint64_t)n * ((1ull << 34) + 2) + merges;
  wacc_finalize_kernel<<<1, kDotThreads, 0, s>>>(partials, nb, out, take_sqrt, err, G);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  int64_t gx = (n + 4 * kDotThreads - 1) / (4 * kDotThreads);
  const int64_t gmax = 2 * (int64_t)device_sm_count();
  if (gx > gmax) gx = gmax;
  qdot_exact_kernel<<<(unsigned)gx, kDotThreads, 0, s>>>(n, x, incx, y, incy, G, out, take_sqrt);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// qaxpy: y_i = fma(alpha, x_i, y_i), one rounding per element; bit-exact
// with Sleef_fmaq1_u05(alpha, x[i], y[i]) (level1.hpp:150,156,207).
// ---------------------------------------------------------------------------
constexpr int kAxpyThreads = 256;

__global__ void __launch_bounds__(kAxpyThreads)
    qaxpy_kernel(int64_t n, q128 alpha, const q128* __restrict__ x, int64_t incx,
                 q128* __restrict__ y, int64_t incy) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    q128 xv = ld_stream(x + i * incx);
    q128 yv = ld_stream(y + i * incy);
    q128 r = q_fma(alpha, xv, yv);
    ulonglong2 v;
    v.x = r.lo;
    v.y = r.hi;
    __stcs(reinterpret_cast<ulonglong2*>(y + i * incy), v);
  }
}

cudaError_t launch_axpy(int64_t n, q128 alpha, const q128* x, int64_t incx, q128* y, int64_t incy,
                        cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  int64_t want = (n + kAxpyThreads - 1) / kAxpyThreads;
  int64_t cap = (int64_t)device_sm_count() * 8;
  int64_t nb = want < cap ? want : cap;
  qaxpy_kernel<<<(unsigned)nb, kAxpyThreads, 0, s>>>(n, alpha, x, incx, y, incy);
  return cudaGetLastError();
}

}  // namespace qb
