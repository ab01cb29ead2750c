// Ozaki-split qgemv on the 5th-generation tensor cores (tcgen05, sm_103a),
// correctly rounded.
//
// Replaces QuadBLAS::gemv_row_major / gemv_col_major
// (include/quadblas/algorithms/level2.hpp:15-100) for large matrices: each
// y_i is the correctly rounded exact sum_j A(i,j) x_j followed by the
// reference epilogue y_i = fma(alpha, sum, beta * y_i) (level2.hpp:48),
// bit-identical to the soft-float kernels of level2.cu.
//
// The arithmetic (ozgemv.cuh): per chunk of 32 columns every element is
// scaled by its row's largest exponent and cut into 18 balanced 8-bit
// digits; the digit products run on tcgen05.mma kind::f16 (fp16 digits, fp32
// accumulators in tensor memory, exact), one 128 x 32 accumulator per
// (128-row tile, chunk) whose column g is the diagonal sum
// D_g = sum_j sum_{t+u=g} d_t(A(i,j)) d_u(x_j); the chunk's value
// T * 2^(E+F-162) and an error bound 2^(E+F-133) are added into a wide
// accumulator per row.  A finish kernel merges the pieces of each row,
// certifies the rounding against the accumulated bound and lists the rows
// it cannot certify (wide exponent spreads inside a chunk, NaN or infinity)
// for the exact recomputation of level2.cu.
//
// Kernels:
//   og_x_split_kernel : x's chunk exponents F_c (NaN / inf marked) and its
//                       digits as the MMA's B operand, one 1792-byte tile per
//                       16 columns; resets the list of uncertified rows
//   og_gemv_kernel    : persistent, one CTA per SM over a balanced range of
//                       (row tile, chunk) items, warp-specialised:
//                       warps 0-7  split A (two threads per row, 8 columns
//                                  each per 16-column k-step): load, scale,
//                                  byte-select digits, st.shared into a
//                                  double-buffered operand stage;
//                       warp 8     issues 18 tcgen05.mma (M=128, N=32,
//                                  K=16) per k-step, one per A digit plane
//                                  t, with B = x's planes shifted down by t
//                                  (a descriptor offset), so the one
//                                  accumulator collects every diagonal;
//                       warps 9-12 read the accumulator (tcgen05.ld), fold
//                                  the diagonals and add into the row's
//                                  wide accumulator; one partial per
//                                  (row, CTA range).
//                       Every mbarrier wait is bounded (1 s): on timeout the
//                       kernel records an error and returns, after draining
//                       its MMAs and freeing tensor memory.
//   og_finish_kernel  : per row: merge the partials in order, certify, apply
//                       the epilogue or list the row.
//
// Shared memory of one operand stage (no swizzle, K-major core matrices of
// 8 rows x 16 bytes): 18 A planes of 128 rows x 16 columns (plane t at
// t * 4096, columns 8..15 at +2048, row r at (r/8)*128 + (r%8)*16), then the
// B tile: 56 rows x 16 columns (row 17 + u holds x's plane u, the rest zero;
// columns 8..15 at +896), so B for plane t starts at row 17 - t.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "exact.cuh"
#include "gemv_rows.cuh"
#include "kernels.h"
#include "ozgemv.cuh"
#include "reduce.cuh"
#include "umma.cuh"

namespace qb {

constexpr int kOgRows = 128;                 // rows per tile (MMA M)
constexpr int kOgSplitWarps = 8;
constexpr int kOgEpiWarps = 4;
constexpr int kOgMmaWarp = kOgSplitWarps;    // warp 8: tcgen05.mma and the TMA loads of A
constexpr int kOgThreads = (kOgSplitWarps + 1 + kOgEpiWarps) * 32;  // 416
constexpr int kOgKStep = 16;                 // columns per MMA (K)
constexpr int kOgPlaneBytes = kOgRows * kOgKStep * 2;  // 4096
constexpr int kOgALbo = kOgPlaneBytes / 2;   // 2048: core matrices of columns 8..15
constexpr int kOgXRows = 56;
constexpr int kOgXLbo = kOgXRows * 16;       // 896
constexpr int kOgXBytes = 2 * kOgXLbo;       // 1792 per k-step
constexpr int kOgXBase = kOgPlanes - 1;      // x plane u at B row 17 + u
constexpr int kOgDigitBytes = kOgPlanes * kOgPlaneBytes + kOgXBytes;  // 75520: one operand stage
constexpr int kOgSlotBytes = kOgRows * kOgKStep * 16;  // 32768: A elements of one k-step
constexpr int kOgSlots = 4;                  // TMA ring: two chunks
constexpr int kOgExpSlots = 4;
constexpr int kOgTmemCols = 64;              // two 32-column accumulators
constexpr int kOgXSpecial = 0x7FFFFFFF;      // x chunk holding NaN or inf
constexpr int kOgNoGmax = 2 * kOgNoExp;
// kind::f16, fp16 A and B (K-major), fp32 D, N = 32, M = 128
constexpr uint32_t kOgIdesc = (1u << 4) | ((32u >> 3) << 17) | ((uint32_t)(kOgRows >> 4) << 24);
// barriers: full[4] (TMA), ready, free (operand stage), tfull[2], tempty[2], exp[4], drain
constexpr int kOgBars = kOgSlots + 2 + 4 + kOgExpSlots + 1;
constexpr size_t kOgSmem = 1024 + (size_t)kOgSlots * kOgSlotBytes + kOgDigitBytes + kOgExpSlots * kOgRows * 4 +
                           kOgBars * 8 + 16;

struct OgPartial {
  wacc acc;
  int32_t gmax;   // largest E + F over chunks with a nonzero x element
  uint32_t nch;   // chunks added
  uint32_t spec;  // a NaN or infinity was seen
  uint32_t pad;
};

struct OgParams {
  int64_t m, n;
  const uint8_t* xdig;      // [2 * nchunks][kOgXBytes]
  const int32_t* xexp;      // [nchunks]: F_c, kOgNoExp, or kOgXSpecial
  int64_t tiles, nchunks, work;  // work = tiles * nchunks items
  int segs;                 // partial slots per tile
  OgPartial* part;          // [tiles][segs][128]
  int* err;
};

// First item of CTA b's range, and the CTA whose range holds item X.
QB_HD int64_t og_range_begin(int64_t work, int64_t G, int64_t b) { return work * b / G; }
QB_HD int64_t og_cta_of(int64_t work, int64_t G, int64_t X) { return ((X + 1) * G + work - 1) / work - 1; }

// ---------------------------------------------------------------------------
// x digits
// ---------------------------------------------------------------------------
// One warp per chunk of 32 elements of x.
__global__ void __launch_bounds__(256)
    og_x_split_kernel(int64_t n, int64_t nchunks, const q128* __restrict__ x, int64_t incx,
                      uint8_t* __restrict__ xdig, int32_t* __restrict__ xexp, RowList* __restrict__ L) {
  if (blockIdx.x == 0 && threadIdx.x == 0) L->count = 0;
  const int lane = threadIdx.x & 31;
  const int64_t c = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (c >= nchunks) return;
  const int64_t j = c * kOgChunk + lane;
  q128 v;
  v.lo = v.hi = 0;
  if (j < n) v = ld_cached(x + j * incx);
  const uint32_t top = (uint32_t)(v.hi >> 32);
  const bool special = og_special_top(top);
  const bool nonzero = ((v.hi & 0x7FFFFFFFFFFFFFFFull) | v.lo) != 0;
  int f = (nonzero && !special) ? og_lead_top(top) : kOgNoExp;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) f = max(f, __shfl_xor_sync(0xFFFFFFFFu, f, o));
  const bool any_special = __any_sync(0xFFFFFFFFu, special);
  if (lane == 0) xexp[c] = any_special ? kOgXSpecial : f;
  uint32_t W[5];
  og_window((uint32_t)v.lo, (uint32_t)(v.lo >> 32), (uint32_t)v.hi, top, f == kOgNoExp ? -16382 : f, W);
  // B tile of k-step 2c + lane/16, column lane%16
  uint8_t* tile = xdig + (size_t)(2 * c + (lane >> 4)) * kOgXBytes;
  const int kk = lane & 15;
  __half* col = reinterpret_cast<__half*>(tile + (kk >> 3) * kOgXLbo + (kk & 7) * 2);
  for (int rho = 0; rho < kOgXRows; ++rho) {
    const int u = rho - kOgXBase;
    const int d = (u >= 0 && u < kOgPlanes) ? og_digit(W, u) : 0;
    col[rho * 8] = __int2half_rn(d);  // rows are 16 bytes apart
  }
}

// ---------------------------------------------------------------------------
// Main kernel
// ---------------------------------------------------------------------------
__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d)
               : "memory");
}

__device__ __forceinline__ uint4 ld_shared_v4(uint32_t addr) {
  uint4 v;
  asm volatile("ld.shared.v4.b32 {%0, %1, %2, %3}, [%4];" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "r"(addr));
  return v;
}

__device__ __forceinline__ uint32_t ld_shared_u32(uint32_t addr) {
  uint32_t v;
  asm volatile("ld.shared.b32 %0, [%1];" : "=r"(v) : "r"(addr));
  return v;
}

// Two digits of plane t (byte 17 - t of the windows of two elements) as an
// fp16 pair: (1024 + byte) - 1152.
template <int kT>
__device__ __forceinline__ uint32_t og_digit_pair(const uint32_t (&Wa)[5], const uint32_t (&Wb)[5]) {
  constexpr int beta = 17 - kT, w = beta >> 2, by = beta & 3;
  const uint32_t p = __byte_perm(Wa[w], Wb[w], (uint32_t)(by | ((4 + by) << 4)));
  uint32_t q = __byte_perm(p, 0x64646464u, 0x5140u);
  uint32_t bias = 0xE480E480u;  // fp16 -1152 twice
  __half2 h = __hadd2(*reinterpret_cast<__half2*>(&q), *reinterpret_cast<__half2*>(&bias));
  return *reinterpret_cast<uint32_t*>(&h);
}

template <int kT>
__device__ __forceinline__ void og_store_plane(uint32_t addr, const uint32_t (&W)[8][5]) {
  st_shared_v4(addr + kT * kOgPlaneBytes, og_digit_pair<kT>(W[0], W[1]), og_digit_pair<kT>(W[2], W[3]),
               og_digit_pair<kT>(W[4], W[5]), og_digit_pair<kT>(W[6], W[7]));
  if constexpr (kT + 1 < kOgPlanes) og_store_plane<kT + 1>(addr, W);
}

// A's elements of one k-step arrive by TMA (128-byte swizzle: the 16-byte
// piece p of a 128-byte smem row q sits at piece p ^ (q % 8)).
//   row-major A: two boxes of 128 rows x 8 columns (columns 8h..8h+7 at
//                h * 16384; element (r, 8h + i) at r * 128 + piece i)
//   column-major A: sixteen boxes of 8 rows x 16 columns (rows 8g..8g+7 at
//                g * 2048; element (8g + e, j) at j * 128 + piece e)
// Offset of thread (row r, half h)'s element i within a slot:
template <bool kRowMajor>
__device__ __forceinline__ uint32_t og_elem_offset(int r, int h, int i) {
  if (kRowMajor) return (uint32_t)(h * 16384 + r * 128 + ((i ^ (r & 7)) << 4));
  const int j = 8 * h + i;
  return (uint32_t)((r >> 3) * 2048 + j * 128 + (((r & 7) ^ (j & 7)) << 4));
}

// 13 warps: four share one SM sub-partition's 16384 registers, so at most
// 128 registers per thread; one CTA per SM.
template <bool kRowMajor>
__global__ void __launch_bounds__(kOgThreads, 1)
    og_gemv_kernel(const __grid_constant__ CUtensorMap tmA, OgParams P) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;  // slots: 1024-byte aligned for the swizzle
  uint8_t* gbase = smem_raw + (base - raw);
  const uint32_t dstage = base + kOgSlots * kOgSlotBytes;  // digit planes + x tile
  int32_t* exps = reinterpret_cast<int32_t*>(gbase + kOgSlots * kOgSlotBytes + kOgDigitBytes);  // [4][128]
  const uint32_t bar0 = dstage + kOgDigitBytes + kOgExpSlots * kOgRows * 4;
  auto full_bar = [&](int s) { return bar0 + 8u * s; };
  const uint32_t ready_bar = bar0 + 8u * kOgSlots, free_bar = ready_bar + 8u;
  auto tfull_bar = [&](int b) { return bar0 + 8u * (kOgSlots + 2 + b); };
  auto tempty_bar = [&](int b) { return bar0 + 8u * (kOgSlots + 4 + b); };
  auto exp_bar = [&](int s) { return bar0 + 8u * (kOgSlots + 6 + s); };
  const uint32_t drain_bar = bar0 + 8u * (kOgBars - 1);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(gbase + (bar0 - base) + kOgBars * 8);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kOgSlots; ++s) mbar_init(full_bar(s), 1);
    mbar_init(ready_bar, kOgSplitWarps);
    mbar_init(free_bar, 1);
    for (int b = 0; b < 2; ++b) {
      mbar_init(tfull_bar(b), 1);
      mbar_init(tempty_bar(b), kOgEpiWarps);
    }
    for (int s = 0; s < kOgExpSlots; ++s) mbar_init(exp_bar(s), 1);
    mbar_init(drain_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == kOgMmaWarp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kOgTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  const int64_t G = gridDim.x;
  const int64_t w0 = og_range_begin(P.work, G, blockIdx.x), w1 = og_range_begin(P.work, G, blockIdx.x + 1);
  const uint32_t nks = (uint32_t)(2 * (w1 - w0));  // k-steps of this CTA
  bool ok = true;

  if (warp < kOgSplitWarps) {
    // ---------------- split: two threads per row ----------------
    const int r = warp * 16 + (lane >> 1), h = lane & 1;
    const int tid = threadIdx.x;
    uint32_t off[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) off[i] = og_elem_offset<kRowMajor>(r, h, i);
    uint32_t q = 0, it = 0;
    for (int64_t w = w0; w < w1 && ok; ++w, ++it) {
      // both k-steps of the chunk are needed for its row exponents
      if (!mbar_wait(full_bar(q & 3), (q >> 2) & 1u) || !mbar_wait(full_bar((q + 1) & 3), ((q + 1) >> 2) & 1u)) {
        ok = false;
        break;
      }
      int E = -16382;
      uint32_t sp = 0;
#pragma unroll
      for (int ks = 0; ks < 2; ++ks) {
        const uint32_t slot = base + ((q + ks) & 3) * kOgSlotBytes;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const uint32_t top = ld_shared_u32(slot + off[i] + 12);
          E = max(E, og_lead_top(top));
          sp |= og_special_top(top) ? 1u : 0u;
        }
      }
      E = max(E, __shfl_xor_sync(0xFFFFFFFFu, E, 1));
      sp |= __shfl_xor_sync(0xFFFFFFFFu, sp, 1);
      const int64_t c = w % P.nchunks;
#pragma unroll 1
      for (int ks = 0; ks < 2; ++ks, ++q) {
        uint4 xv = make_uint4(0, 0, 0, 0);
        if (tid < kOgXBytes / 16)
          xv = __ldg(reinterpret_cast<const uint4*>(P.xdig + (size_t)(2 * c + ks) * kOgXBytes) + tid);
        const uint32_t slot = base + (q & 3) * kOgSlotBytes;
        uint32_t W[8][5];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const uint4 v = ld_shared_v4(slot + off[i]);
          og_window(v.x, v.y, v.z, v.w, E, W[i]);
        }
        // the operand stage is free once the previous k-step's MMAs completed
        if (!mbar_wait(free_bar, (q & 1u) ^ 1u)) {
          ok = false;
          break;
        }
        if (ks == 0 && h == 0) exps[(it & 3) * kOgRows + r] = (E << 1) | (int)sp;
        og_store_plane<0>(dstage + h * kOgALbo + (r >> 3) * 128 + (r & 7) * 16, W);
        if (tid < kOgXBytes / 16)
          st_shared_v4(dstage + kOgPlanes * kOgPlaneBytes + tid * 16, xv.x, xv.y, xv.z, xv.w);
        fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(ready_bar);
      }
    }
    if (!ok && lane == 0) atomicExch(P.err, 1);
  } else if (warp == kOgMmaWarp) {
    // ---------------- TMA loads of A and MMA issue ----------------
    if (lane == 0) {
      auto load_kstep = [&](uint32_t kq) {  // k-step kq of this CTA into slot kq % 4
        const int64_t w = w0 + kq / 2;
        const int64_t tile = w / P.nchunks, c = w % P.nchunks;
        const int col0 = (int)(c * kOgChunk + (kq & 1) * kOgKStep);
        const uint32_t slot = base + (kq & 3) * kOgSlotBytes, bar = full_bar(kq & 3);
        mbar_expect_tx(bar, kOgSlotBytes);
        if (kRowMajor) {
          for (int hh = 0; hh < 2; ++hh)
            tma_load_2d(slot + hh * 16384, &tmA, bar, 4 * (col0 + 8 * hh), (int)(tile * kOgRows));
        } else {
          for (int g = 0; g < kOgRows / 8; ++g)
            tma_load_2d(slot + g * 2048, &tmA, bar, 4 * (int)(tile * kOgRows + 8 * g), col0);
        }
      };
      uint32_t issued = 0;
      for (; issued < nks && issued < (uint32_t)kOgSlots; ++issued) load_kstep(issued);
      uint32_t q = 0, it = 0;
      bool any_mma = false;
      for (int64_t w = w0; w < w1 && ok; ++w, ++it) {
        const int tb = it & 1;
        if (!mbar_wait(tempty_bar(tb), ((it >> 1) & 1u) ^ 1u)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        for (int ks = 0; ks < 2 && ok; ++ks, ++q) {
          if (!mbar_wait(ready_bar, q & 1u)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          if (ks == 0) mbar_arrive(exp_bar(it & 3));  // this item's row exponents are written
          // slot q % 4 has been read: refill it with k-step q + 4
          if (issued < nks) load_kstep(issued++);
          const uint32_t xb = dstage + kOgPlanes * kOgPlaneBytes;
#pragma unroll
          for (int t = 0; t < kOgPlanes; ++t) {
            const uint64_t da = smem_desc_noswizzle(dstage + t * kOgPlaneBytes, kOgALbo, 128);
            const uint64_t db = smem_desc_noswizzle(xb + (kOgXBase - t) * 16, kOgXLbo, 128);
            mma_f16kind(tmem + (uint32_t)(tb * 32), da, db, kOgIdesc, (ks | t) ? 1u : 0u);
          }
          any_mma = true;
          mma_commit(free_bar);
        }
        if (!ok) break;
        mma_commit(tfull_bar(tb));
      }
      if (!ok) {
        atomicExch(P.err, 1);
        if (any_mma) {
          mma_commit(drain_bar);
          mbar_wait(drain_bar, 0);
        }
        // copies still in flight: the last (up to) four issued
        for (uint32_t j = (issued > (uint32_t)kOgSlots ? issued - kOgSlots : 0); j < issued; ++j)
          mbar_wait(full_bar(j & 3), (j >> 2) & 1u);
      }
    }
  } else {
    // ---------------- epilogue: thread per row ----------------
    const int quad = warp & 3;
    const int rit = quad * 32 + lane;
    wacc acc;
    wacc_init(acc);
    int gmax = kOgNoGmax;
    uint32_t nch = 0, spec = 0;
    int64_t cur = -1;
    auto flush = [&](int64_t tile) {
      const int64_t k = (int64_t)blockIdx.x - og_cta_of(P.work, G, tile * P.nchunks);
      OgPartial& o = P.part[((size_t)tile * P.segs + (size_t)k) * kOgRows + rit];
      o.acc = acc;
      o.gmax = gmax;
      o.nch = nch;
      o.spec = spec;
      o.pad = 0;
    };
    uint32_t it = 0;
    for (int64_t w = w0; w < w1 && ok; ++w, ++it) {
      const int64_t tile = w / P.nchunks, c = w % P.nchunks;
      if (tile != cur) {
        if (cur >= 0) flush(cur);
        wacc_init(acc);
        gmax = kOgNoGmax;
        nch = spec = 0;
        cur = tile;
      }
      const int tb = it & 1;
      if (!mbar_wait(exp_bar(it & 3), (it >> 2) & 1u)) {
        ok = false;
        break;
      }
      const int ev = exps[(it & 3) * kOgRows + rit];
      if (!mbar_wait(tfull_bar(tb), (it >> 1) & 1u)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      uint32_t rr[32];
      tmem_ld32(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(tb * 32), rr);
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(tempty_bar(tb));
      const int E = ev >> 1;
      spec |= (uint32_t)ev & 1u;
      const int F = __ldg(P.xexp + c);
      if (F == kOgXSpecial) {
        spec = 1;
      } else if (F != kOgNoExp) {
        int32_t D[kOgDiags];
#pragma unroll
        for (int g = 0; g < kOgDiags; ++g) D[g] = __float2int_rn(__uint_as_float(rr[g]));
        uint32_t T[6];
        og_fold(D, T);
        og_wacc_add(acc, T, E + F - kOgFoldShift);
        gmax = max(gmax, E + F);
      }
      ++nch;
    }
    if (ok && cur >= 0) flush(cur);
    if (!ok && lane == 0) atomicExch(P.err, 1);
  }

  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == kOgMmaWarp) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kOgTmemCols)
                 : "memory");
  }
}

// ---------------------------------------------------------------------------
// Finish
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128)
    og_finish_kernel(int64_t m, int64_t nchunks, int64_t work, int64_t G, int segs,
                     const OgPartial* __restrict__ part, const int* __restrict__ err, q128 alpha, q128 beta,
                     q128* __restrict__ y, int64_t incy, RowList* __restrict__ L) {
  const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= m) return;
  const int64_t tile = row / kOgRows, rit = row % kOgRows;
  const int64_t X0 = tile * nchunks, X1 = X0 + nchunks;
  const int64_t bf = og_cta_of(work, G, X0), bl = og_cta_of(work, G, X1 - 1);
  wacc acc;
  wacc_init(acc);
  int gmax = kOgNoGmax;
  uint32_t nch = 0, spec = *err != 0;  // a timed-out kernel leaves every row to the exact pass
  uint64_t merges = 0;
  for (int64_t b = bf; b <= bl; ++b) {
    const int64_t r0 = og_range_begin(work, G, b), r1 = og_range_begin(work, G, b + 1);
    if (r1 <= X0 || r0 >= X1 || r0 == r1) continue;
    const OgPartial& p = part[((size_t)tile * segs + (size_t)(b - bf)) * kOgRows + rit];
    wacc_merge(acc, p.acc);
    gmax = max(gmax, p.gmax);
    nch += p.nch;
    spec |= p.spec;
    ++merges;
  }
  q128* yp = y + row * incy;
  if (spec || (gmax != kOgNoGmax && acc.e == kWaccEmptyExp)) {
    L->row[atomicAdd(&L->count, 1u)] = row;
    return;
  }
  const uint64_t e = gmax == kOgNoGmax ? 0 : og_row_error(acc, nch, gmax, 3 * merges + 3);
  gemv_finish_row(alpha, acc, e, beta, yp, row, L);
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
static size_t og_round256(size_t b) { return (b + 255) & ~(size_t)255; }

struct OgLayout {
  int64_t tiles, nchunks, work, G;
  int segs;
  size_t xdig, xexp, part, err, total;
};

static OgLayout og_layout(int64_t m, int64_t n) {
  OgLayout L;
  L.tiles = (m + kOgRows - 1) / kOgRows;
  L.nchunks = (n + kOgChunk - 1) / kOgChunk;
  L.work = L.tiles * L.nchunks;
  const int64_t sms = device_sm_count();
  L.G = L.work < sms ? L.work : sms;
  L.segs = 1;  // CTAs whose ranges meet one tile, at most
  for (int64_t t = 0; t < L.tiles; ++t) {
    const int64_t k = og_cta_of(L.work, L.G, (t + 1) * L.nchunks - 1) - og_cta_of(L.work, L.G, t * L.nchunks) + 1;
    if (k > L.segs) L.segs = (int)k;
  }
  L.xdig = 0;
  L.xexp = L.xdig + og_round256((size_t)L.nchunks * 2 * kOgXBytes);
  L.err = L.xexp + og_round256((size_t)L.nchunks * 4);
  L.part = L.err + 256;
  L.total = L.part + og_round256((size_t)L.tiles * L.segs * kOgRows * sizeof(OgPartial));
  return L;
}

size_t gemv_ozaki_scratch_bytes(int64_t m, int64_t n) {
  if (m <= 0 || n <= 0) return 0;
  return og_layout(m, n).total;
}

cudaError_t launch_gemv_ozaki(int64_t m, int64_t n, q128 alpha, MatView A, const q128* x, int64_t incx,
                              q128 beta, q128* y, int64_t incy, RowList* list, void* scratch, cudaStream_t s) {
  const bool row_major = A.sj == 1;
  const int64_t ld = row_major ? A.si : A.sj;
  if (!row_major && A.si != 1) return cudaErrorInvalidValue;
  // A as 32-bit words, [rows][4 * cols] (row-major) or [cols][4 * rows]
  CUtensorMap map;
  {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return cudaErrorNotSupported;
    const int64_t inner = row_major ? n : m, outer = row_major ? m : n;
    cuuint64_t dims[2] = {(cuuint64_t)(4 * inner), (cuuint64_t)outer};
    cuuint64_t strides[1] = {(cuuint64_t)ld * 16};
    cuuint32_t box[2] = {32, row_major ? (cuuint32_t)kOgRows : (cuuint32_t)kOgKStep};
    cuuint32_t estr[2] = {1, 1};
    if (fn(&map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, const_cast<q128*>(A.p), dims, strides, box, estr,
           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return cudaErrorInvalidValue;
  }
  const OgLayout Lo = og_layout(m, n);
  char* base = static_cast<char*>(scratch);
  OgParams P;
  P.m = m;
  P.n = n;
  P.xdig = reinterpret_cast<uint8_t*>(base + Lo.xdig);
  P.xexp = reinterpret_cast<int32_t*>(base + Lo.xexp);
  P.tiles = Lo.tiles;
  P.nchunks = Lo.nchunks;
  P.work = Lo.work;
  P.segs = Lo.segs;
  P.part = reinterpret_cast<OgPartial*>(base + Lo.part);
  P.err = reinterpret_cast<int*>(base + Lo.err);
  cudaError_t e = cudaMemsetAsync(P.err, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  {
    const int64_t warps = Lo.nchunks, per_block = 8;
    og_x_split_kernel<<<(unsigned)((warps + per_block - 1) / per_block), 256, 0, s>>>(
        n, Lo.nchunks, x, incx, const_cast<uint8_t*>(P.xdig), const_cast<int32_t*>(P.xexp), list);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  static bool attr = false;
  if (!attr) {
    if ((e = cudaFuncSetAttribute(og_gemv_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kOgSmem)) != cudaSuccess ||
        (e = cudaFuncSetAttribute(og_gemv_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kOgSmem)) != cudaSuccess)
      return e;
    attr = true;
  }
  if (row_major)
    og_gemv_kernel<true><<<(unsigned)Lo.G, kOgThreads, kOgSmem, s>>>(map, P);
  else
    og_gemv_kernel<false><<<(unsigned)Lo.G, kOgThreads, kOgSmem, s>>>(map, P);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  og_finish_kernel<<<(unsigned)((m + 127) / 128), 128, 0, s>>>(m, Lo.nchunks, Lo.work, Lo.G, Lo.segs, P.part,
                                                              P.err, alpha, beta, y, incy, list);
  return cudaGetLastError();
}

}  // namespace qb
