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
//                       digits as the MMA's B operand, one 1536-byte tile per
//                       8-column k-step; resets the list of uncertified rows
//   og_gemv_kernel    : persistent, one CTA per SM over a balanced range of
//                       (row tile, chunk) items, 22 warps, warp-specialised:
//                       warps 0-15 split A: thread per row (its tensor-memory
//                                  lane; warp % 4 is the lane quadrant),
//                                  two columns per 8-column k-step (warp / 4
//                                  picks which); the four warps of a quadrant
//                                  exchange the row's largest exponent, then
//                                  each builds its elements' windows, turns
//                                  digit pairs into fp16 pairs (byte select +
//                                  HFMA2) and writes them to the A operand
//                                  stage in tensor memory (tcgen05.st);
//                       warp 16    issues 9 tcgen05.mma (M=128, N=32,
//                                  K=16: 8 elements x 2 digit planes) per
//                                  k-step, one per plane pair p, A from
//                                  tensor memory, B = x's tile read 16 - 2p
//                                  rows down (a descriptor offset), so the
//                                  one accumulator collects every diagonal;
//                       warp 17    TMA loads of A's k-steps into a ring of
//                                  12 shared-memory slots (16 KB each,
//                                  128-byte swizzle), each with a bulk
//                                  copy of x's B tile for the k-step into
//                                  a ring of 16 B slots (a B slot is
//                                  reused once the MMAs that read it
//                                  completed);
//                       warps 18-21 read the accumulator (tcgen05.ld), fold
//                                  the diagonals and add into the row's
//                                  wide accumulator; one partial per
//                                  (row, CTA range).
//                       Four operand stages and four accumulators are in
//                       flight.  Every mbarrier wait is bounded (1 s): on
//                       timeout the kernel records an error and returns,
//                       after waiting (bounded) for its copies and MMAs and
//                       freeing tensor memory.
//   og_finish_kernel  : per row: merge the partials in order, certify, apply
//                       the epilogue or list the row.
//
// A reaches shared memory in one of three TMA layouts (og_elem_offset):
// row-major A as a 2-D box of 128 rows x 8 columns; column-major A with m a
// multiple of 8 as one 3-D box (8-row groups x columns); other column-major
// A as sixteen 2-D boxes of 8 rows.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <atomic>

#include "exact.cuh"
#include "gemv_rows.cuh"
#include "kernels.h"
#include "ozgemv.cuh"
#include "reduce.cuh"
#include "umma.cuh"

namespace qb {

constexpr int kOgRows = 128;                 // rows per tile (MMA M)
constexpr int kOgSplitWarps = 16;            // four per tensor-memory lane quadrant
constexpr int kOgEpiWarps = 4;
constexpr int kOgMmaWarp = kOgSplitWarps;    // warp 16: tcgen05.mma
constexpr int kOgLoadWarp = kOgSplitWarps + 1;  // warp 17: TMA loads of A
constexpr int kOgThreads = (kOgSplitWarps + 2 + kOgEpiWarps) * 32;  // 704
constexpr int kOgKStep = 8;                  // columns per k-step: MMA K = 8 elements x 2 planes
constexpr int kOgKSteps = kOgChunk / kOgKStep;  // 4 per chunk
constexpr int kOgPairs = kOgPlanes / 2;     // 9 plane pairs: one MMA each per k-step
// tensor memory: four 32-column accumulators (items in flight between the
// MMAs and the epilogue), then the A operand stages: 9 tiles of 8 columns
// (128 lanes x 16 fp16 values) per k-step
constexpr int kOgAccBufs = 4;
constexpr int kOgAccCols = kOgAccBufs * 32;  // 128
constexpr int kOgTileCols = 8;
constexpr int kOgStageCols = kOgPairs * kOgTileCols;  // 72
constexpr int kOgStages = 4;                 // operand stages in flight
constexpr int kOgTmemCols = 512;             // 128 + 4 * 72 = 416 used
constexpr int kOgXRows = 48;                 // B rows: diagonal g of pair p at row g + 16 - 2p
constexpr int kOgXLbo = kOgXRows * 16;       // 768
constexpr int kOgXBytes = 2 * kOgXLbo;       // 1536: B operand of one k-step
constexpr int kOgSlotBytes = kOgRows * kOgKStep * 16;  // 16384: A elements of one k-step
constexpr int kOgSlots = 12;                 // TMA ring: three chunks
constexpr int kOgXSlots = 16;                // x's B tiles: k-step q in slot q % 16, reused after q's MMAs
constexpr int kOgExpSlots = 8;
constexpr int kOgXSpecial = 0x7FFFFFFF;      // x chunk holding NaN or inf
constexpr int kOgNoGmax = 2 * kOgNoExp;
// kind::f16, fp16 A and B (K-major), fp32 D, N = 32, M = 128
constexpr uint32_t kOgIdesc = (1u << 4) | ((32u >> 3) << 17) | ((uint32_t)(kOgRows >> 4) << 24);
// barriers: full[slots], empty[slots] (TMA ring: A elements and x's B tile), ready[stages],
// free[stages], tfull[accs], tempty[accs], exp[8], rowmax[2][4] (the four split warps of a
// lane quadrant), drain, bempty[x slots] (the MMAs reading a B tile completed)
constexpr int kOgBars = 2 * kOgSlots + 2 * kOgStages + 2 * kOgAccBufs + kOgExpSlots + 8 + 1 + kOgXSlots;
constexpr size_t kOgSmem = 1024 + (size_t)kOgSlots * kOgSlotBytes + (size_t)kOgXSlots * kOgXBytes +
                           kOgExpSlots * kOgRows * 4 + 2 * 4 * kOgRows * 4 + kOgBars * 8 + 16;
static_assert(kOgSmem <= 232448, "og_gemv_kernel shared memory");

struct OgPartial {
  wacc acc;
  int32_t gmax;   // largest E + F over chunks with a nonzero x element
  uint32_t nch;   // chunks added
  uint32_t spec;  // a NaN or infinity was seen
  uint32_t pad;
};

struct OgParams {
  int64_t m, n;
  const uint8_t* xdig;      // [4 * nchunks][kOgXBytes]
  const int32_t* xexp;      // [nchunks]: F_c, kOgNoExp, or kOgXSpecial
  int64_t tiles, nchunks, work;  // work = tiles * nchunks items
  int segs;                 // partial slots per tile
  OgPartial* part;          // [tiles][segs][128]
  int* err;
  // test hook (quadblas_debug_stall_next_call): pipeline waits give up after
  // wait_ns; withhold = 1 makes the MMA issuer skip the accumulator-full
  // commit of its first item, so that the epilogue's wait runs out
  unsigned long long wait_ns;
  int withhold;
};

// ---------------------------------------------------------------------------
// x digits
// ---------------------------------------------------------------------------
// One warp (one block) per chunk of 32 elements of x: F_c, and the B operand
// of each k-step (8 columns): row rho, K = 2 * (column % 8) + tt holds x's
// digit rho - 16 - tt (zero outside 0..17), K-major core matrices (LBO 768);
// the chunk's four tiles are built in shared memory and written with
// 16-byte stores.
__global__ void __launch_bounds__(32)
    og_x_split_kernel(int64_t n, int64_t nchunks, const q128* __restrict__ x, int64_t incx,
                      uint8_t* __restrict__ xdig, int32_t* __restrict__ xexp, RowList* __restrict__ L) {
  __shared__ __align__(16) __half tiles[kOgKSteps * kOgXBytes / 2];
  if (blockIdx.x == 0 && threadIdx.x == 0) L->count = 0;
  const int lane = threadIdx.x;
  const int64_t c = blockIdx.x;
  if (c >= nchunks) return;
  const int64_t j = c * kOgChunk + lane;
  q128 v;
  v.lo = v.hi = 0;
  if (j < n) v = ld_cached(x + j * incx);
  const uint32_t top = (uint32_t)(v.hi >> 32);
  const bool special = og_special_top(top);
  const bool nonzero = ((v.hi & 0x7FFFFFFFFFFFFFFFull) | v.lo) != 0;
  int f = nonzero ? og_lead_top(top) : kOgNoExp;  // chunks with NaN / inf are marked below
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) f = max(f, __shfl_xor_sync(0xFFFFFFFFu, f, o));
  const bool any_special = __any_sync(0xFFFFFFFFu, special);
  if (lane == 0) xexp[c] = any_special ? kOgXSpecial : f;
  uint32_t W[5];
  og_window((uint32_t)v.lo, (uint32_t)(v.lo >> 32), (uint32_t)v.hi, top, f == kOgNoExp ? -16382 : f, W);
  const uint32_t neg = top >> 31;
  __half* tile = tiles + (lane >> 3) * (kOgXBytes / 2);
  for (int tt = 0; tt < 2; ++tt) {
    const int kk = 2 * (lane & 7) + tt;
    __half* col = tile + (kk >> 3) * (kOgXLbo / 2) + (kk & 7);
    for (int rho = 0; rho < kOgXRows; ++rho) {
      const int u = rho - 16 - tt;
      const int d = (u >= 0 && u < kOgPlanes) ? og_digit(W, u, neg) : 0;
      col[rho * 8] = __int2half_rn(d);  // rows are 16 bytes apart
    }
  }
  __syncwarp();
  const uint4* src = reinterpret_cast<const uint4*>(tiles);
  uint4* dst = reinterpret_cast<uint4*>(xdig + (size_t)(kOgKSteps * c) * kOgXBytes);
  for (int k = lane; k < kOgKSteps * kOgXBytes / 16; k += 32) dst[k] = src[k];
}

// ---------------------------------------------------------------------------
// Main kernel
// ---------------------------------------------------------------------------
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

// Digits 2p and 2p+1 of one element (bytes 17-2p and 16-2p of its window)
// as an fp16 pair: sign * ((1024 + byte) - 1152), with sg = (sign, sign)
// and bs = (-1152 sign, -1152 sign).
template <int kP>
__device__ __forceinline__ uint32_t og_digit_pair(const uint32_t (&W)[5], uint32_t sg, uint32_t bs) {
  constexpr int lo = 16 - 2 * kP, w = lo >> 2, by = lo & 3;
  uint32_t q = __byte_perm(W[w], 0x64646464u, (uint32_t)((by + 1) | (4 << 4) | (by << 8) | (4 << 12)));
  __half2 h = __hfma2(*reinterpret_cast<__half2*>(&q), *reinterpret_cast<__half2*>(&sg),
                      *reinterpret_cast<__half2*>(&bs));
  return *reinterpret_cast<uint32_t*>(&h);
}

// The nine digit pairs of two elements into the nine A tiles of a stage
// (tensor memory columns 8p + 2g, 8p + 2g + 1 of this thread's lane).
template <int kP>
__device__ __forceinline__ void og_store_pairs(uint32_t taddr, const uint32_t (&W)[2][5], const uint32_t (&sg)[2],
                                               const uint32_t (&bs)[2]) {
  tmem_st2(taddr + kP * kOgTileCols, og_digit_pair<kP>(W[0], sg[0], bs[0]), og_digit_pair<kP>(W[1], sg[1], bs[1]));
  if constexpr (kP + 1 < kOgPairs) og_store_pairs<kP + 1>(taddr, W, sg, bs);
}

// A's elements of one k-step arrive by TMA (128-byte swizzle: the 16-byte
// piece p of a 128-byte smem row q sits at piece p ^ (q % 8)).
//   kOgRowMajor: one box of 128 rows x 8 columns (element (r, i) at
//                r * 128 + piece i)
//   kOgColGroups: column-major A with m a multiple of 8, as a 3-D tensor
//                (8 rows = 128 bytes, row groups, columns): one box of 16 row
//                groups x 8 columns (element (8g + e, i) at
//                (16 i + g) * 128 + piece e)
//   kOgColBoxes: column-major A otherwise: sixteen 2-D boxes of 8 rows x 8
//                columns (rows 8g..8g+7 at g * 1024; element (8g + e, i) at
//                i * 128 + piece e)
enum : int { kOgRowMajor = 0, kOgColGroups = 1, kOgColBoxes = 2 };

template <int kLayout>
__device__ __forceinline__ uint32_t og_elem_offset(int r, int i) {
  if (kLayout == kOgRowMajor) return (uint32_t)(r * 128 + ((i ^ (r & 7)) << 4));
  const int g = r >> 3, e = r & 7;
  if (kLayout == kOgColGroups) return (uint32_t)((16 * i + g) * 128 + ((e ^ (g & 7)) << 4));
  return (uint32_t)(g * 1024 + i * 128 + ((e ^ i) << 4));
}

// 22 warps: six share one SM sub-partition's 16384 registers, so at most
// 80 registers per thread; one CTA per SM (all 512 tensor-memory columns).
template <int kLayout>
__global__ void __launch_bounds__(kOgThreads, 1)
    og_gemv_kernel(const __grid_constant__ CUtensorMap tmA, OgParams P) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;  // slots: 1024-byte aligned for the swizzle
  uint8_t* gbase = smem_raw + (base - raw);
  const uint32_t xslot0 = base + kOgSlots * kOgSlotBytes;  // x's B tiles
  uint8_t* after = gbase + kOgSlots * kOgSlotBytes + kOgXSlots * kOgXBytes;
  int32_t* exps = reinterpret_cast<int32_t*>(after);                        // [8][128]
  uint32_t* emax = reinterpret_cast<uint32_t*>(after + kOgExpSlots * kOgRows * 4);  // [2][4][128]
  const uint32_t bar0 = base + (uint32_t)(after - gbase) + kOgExpSlots * kOgRows * 4 + 2 * 4 * kOgRows * 4;
  auto full_bar = [&](int s) { return bar0 + 8u * s; };
  auto empty_bar = [&](int s) { return bar0 + 8u * (kOgSlots + s); };
  const uint32_t bar1 = bar0 + 8u * (2 * kOgSlots);
  auto ready_bar = [&](int s) { return bar1 + 8u * s; };
  auto free_bar = [&](int s) { return bar1 + 8u * (kOgStages + s); };
  auto tfull_bar = [&](int b) { return bar1 + 8u * (2 * kOgStages + b); };
  auto tempty_bar = [&](int b) { return bar1 + 8u * (2 * kOgStages + kOgAccBufs + b); };
  auto exp_bar = [&](int s) { return bar1 + 8u * (2 * kOgStages + 2 * kOgAccBufs + s); };
  auto rowmax_bar = [&](int b, int quad) {
    return bar1 + 8u * (2 * kOgStages + 2 * kOgAccBufs + kOgExpSlots + 4 * b + quad);
  };
  const uint32_t drain_bar = bar0 + 8u * (kOgBars - 1 - kOgXSlots);
  auto bempty_bar = [&](int s) { return bar0 + 8u * (kOgBars - kOgXSlots + s); };
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(gbase + (bar0 - base) + kOgBars * 8);
  // k-step q uses TMA slot q % kOgSlots (fill q / kOgSlots) and operand
  // stage q % kOgStages (use q / kOgStages)
  auto slot_of = [](uint32_t kq) { return (int)(kq % kOgSlots); };
  auto xslot_of = [](uint32_t kq) { return (int)(kq % kOgXSlots); };
  auto xfill_parity = [](uint32_t kq) { return (kq / kOgXSlots) & 1u; };
  auto fill_parity = [](uint32_t kq) { return (kq / kOgSlots) & 1u; };
  auto stage_of = [](uint32_t kq) { return (int)(kq % kOgStages); };
  auto use_parity = [](uint32_t kq) { return (kq / kOgStages) & 1u; };

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kOgSlots; ++s) {
      mbar_init(full_bar(s), 1);
      mbar_init(empty_bar(s), kOgSplitWarps);
    }
    for (int s = 0; s < kOgXSlots; ++s) mbar_init(bempty_bar(s), 1);
    for (int s = 0; s < kOgStages; ++s) {
      mbar_init(ready_bar(s), kOgSplitWarps);
      mbar_init(free_bar(s), 1);
    }
    for (int b = 0; b < kOgAccBufs; ++b) {
      mbar_init(tfull_bar(b), 1);
      mbar_init(tempty_bar(b), kOgEpiWarps);
    }
    for (int s = 0; s < kOgExpSlots; ++s) mbar_init(exp_bar(s), 1);
    for (int b = 0; b < 8; ++b) mbar_init(rowmax_bar(b >> 2, b & 3), 4);
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
  const uint32_t nks = (uint32_t)(kOgKSteps * (w1 - w0));  // k-steps of this CTA
  bool ok = true;

  if (warp < kOgSplitWarps) {
    // ---------------- split: thread per row (its tensor-memory lane), 2 columns per k-step ----------------
    const int qd = warp & 3, grp = warp >> 2;  // lane quadrant; columns 2*grp, 2*grp+1 of each k-step
    const int r = qd * 32 + lane;
    const uint32_t off0 = og_elem_offset<kLayout>(r, 2 * grp), off1 = og_elem_offset<kLayout>(r, 2 * grp + 1);
    const uint32_t tlane = tmem + ((uint32_t)(qd * 32) << 16) + kOgAccCols + 2 * grp;
    uint32_t q = 0, it = 0;
    // a chunk's k-steps q .. q + 3 (q a multiple of 4) fill slots s0 .. s0 + 3,
    // s0 = q % kOgSlots, with parity fp = (q / kOgSlots) & 1: kept by counting
    static_assert(kOgSlots % kOgKSteps == 0, "a chunk's k-steps never wrap the slot ring");
    int s0 = 0;
    uint32_t fp = 0;
    for (int64_t w = w0; w < w1 && ok; ++w, ++it) {
      // all k-steps of the chunk are needed for its row exponents
      bool got = true;
#pragma unroll
      for (int ks = 0; ks < kOgKSteps; ++ks) got = got && mbar_wait_ns(full_bar(s0 + ks), fp, P.wait_ns);
      if (!got) {
        ok = false;
        break;
      }
      // largest exponent field: the maximum of top << 1 (sign dropped,
      // exponent first) over the row's 32 columns, which the four warps of
      // this lane quadrant exchange through shared memory (a bounded
      // mbarrier wait, per item parity); the all-ones field marks a NaN or
      // infinity
      uint32_t mx = 0;
#pragma unroll
      for (int ks = 0; ks < kOgKSteps; ++ks) {
        const uint32_t slot = base + (s0 + ks) * kOgSlotBytes;
        mx = max(mx, max(ld_shared_u32(slot + off0 + 12) << 1, ld_shared_u32(slot + off1 + 12) << 1));
      }
      uint32_t* em = emax + (it & 1) * 4 * kOgRows;
      em[grp * kOgRows + r] = mx;
      __syncwarp();
      if (lane == 0) mbar_arrive(rowmax_bar(it & 1, qd));
      if (!mbar_wait_ns(rowmax_bar(it & 1, qd), (it >> 1) & 1u, P.wait_ns)) {
        ok = false;
        break;
      }
      mx = max(max(em[r], em[kOgRows + r]), max(em[2 * kOgRows + r], em[3 * kOgRows + r]));
      const uint32_t bmax = mx >> 17;
      const int E = (int)(bmax > 1u ? bmax : 1u) - 16383;
      const uint32_t sp = bmax == 0x7FFFu ? 1u : 0u;
#pragma unroll 1
      for (int ks = 0; ks < kOgKSteps; ++ks, ++q) {
        const uint32_t slot = base + (s0 + ks) * kOgSlotBytes;
        const uint4 v0 = ld_shared_v4(slot + off0), v1 = ld_shared_v4(slot + off1);
        __syncwarp();
        if (lane == 0) mbar_arrive(empty_bar(s0 + ks));  // this k-step's elements are in registers
        uint32_t W[2][5], sg[2], bs[2];
        const int sh0 = og_shift(E, v0.w), sh1 = og_shift(E, v1.w);
        // the four-word level of the shift only when a lane of the warp needs it
        if (__any_sync(0xFFFFFFFFu, max(sh0, sh1) >= 128)) {
          og_window_s<false>(v0.x, v0.y, v0.z, v0.w, sh0, W[0]);
          og_window_s<false>(v1.x, v1.y, v1.z, v1.w, sh1, W[1]);
        } else {
          og_window_s<true>(v0.x, v0.y, v0.z, v0.w, sh0, W[0]);
          og_window_s<true>(v1.x, v1.y, v1.z, v1.w, sh1, W[1]);
        }
#pragma unroll
        for (int i = 0; i < 2; ++i) {
          const uint32_t neg = (i ? v1.w : v0.w) >> 31;
          sg[i] = 0x3C003C00u + neg * 0x80008000u;  // (+-1, +-1)
          bs[i] = 0xE480E480u - neg * 0x80008000u;  // (-+1152, -+1152)
        }
        const int st = stage_of(q);
        if (!mbar_wait_ns(free_bar(st), use_parity(q) ^ 1u, P.wait_ns)) {  // the MMAs of the stage's last use completed
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (ks == 0 && grp == 0) exps[(it % kOgExpSlots) * kOgRows + r] = (E << 1) | (int)sp;
        og_store_pairs<0>(tlane + st * kOgStageCols, W, sg, bs);
        tmem_st_wait();
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(ready_bar(st));
      }
      s0 += kOgKSteps;
      if (s0 == kOgSlots) {
        s0 = 0;
        fp ^= 1u;
      }
    }
    if (!ok && lane == 0) atomicExch(P.err, 1);
  } else if (warp == kOgLoadWarp) {
    // ---------------- TMA loads of A and x's B tiles into the slot ring ----------------
    if (lane == 0) {
      // TMA cursor: tile, chunk and k-step of the next load, kept by counting
      const int nch = (int)P.nchunks;
      int ld_tile = (int)(w0 / P.nchunks), ld_c = (int)(w0 % P.nchunks), ld_ks = 0;
      auto load_kstep = [&](uint32_t kq) {  // k-step kq of this CTA (loaded in order) into its slot
        const int64_t tile = ld_tile;
        const int col0 = ld_c * kOgChunk + ld_ks * kOgKStep;
        const uint8_t* xsrc = P.xdig + (size_t)(kOgKSteps * ld_c + ld_ks) * kOgXBytes;
        if (++ld_ks == kOgKSteps) {
          ld_ks = 0;
          if (++ld_c == nch) {
            ld_c = 0;
            ++ld_tile;
          }
        }
        const uint32_t slot = base + slot_of(kq) * kOgSlotBytes, bar = full_bar(slot_of(kq));
        mbar_expect_tx(bar, kOgSlotBytes + kOgXBytes);
        bulk_load(xslot0 + xslot_of(kq) * kOgXBytes, xsrc, kOgXBytes, bar);
        if (kLayout == kOgRowMajor) {
          tma_load_2d(slot, &tmA, bar, 4 * col0, (int)(tile * kOgRows));
        } else if (kLayout == kOgColGroups) {
          tma_load_3d(slot, &tmA, bar, 0, (int)(tile * (kOgRows / 8)), col0);
        } else {
          for (int g = 0; g < kOgRows / 8; ++g)
            tma_load_2d(slot + g * 1024, &tmA, bar, 4 * (int)(tile * kOgRows + 8 * g), col0);
        }
      };
      uint32_t issued = 0;
      for (; issued < nks && ok; ++issued) {
        // the split warps released this slot's previous k-step and its MMAs completed
        if (!mbar_wait_ns(empty_bar(slot_of(issued)), fill_parity(issued) ^ 1u, P.wait_ns) ||
            !mbar_wait_ns(bempty_bar(xslot_of(issued)), xfill_parity(issued) ^ 1u, P.wait_ns)) {
          ok = false;
          break;
        }
        load_kstep(issued);
      }
      if (!ok) {
        atomicExch(P.err, 1);
        // copies still in flight: the last (up to) kOgSlots issued
        for (uint32_t j = (issued > (uint32_t)kOgSlots ? issued - kOgSlots : 0); j < issued; ++j)
          mbar_wait(full_bar(slot_of(j)), fill_parity(j));
      }
    }
  } else if (warp == kOgMmaWarp) {
    // ---------------- MMA issue ----------------
    if (lane == 0) {
      const uint64_t db0 = smem_desc_noswizzle(xslot0 + 16 * 16, kOgXLbo, 128);
      uint32_t q = 0, it = 0;
      bool any_mma = false;
      for (int64_t w = w0; w < w1 && ok; ++w, ++it) {
        const int tb = it % kOgAccBufs;
        if (!mbar_wait_ns(tempty_bar(tb), ((it / kOgAccBufs) & 1u) ^ 1u, P.wait_ns)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        for (int ks = 0; ks < kOgKSteps && ok; ++ks, ++q) {
          const int st = stage_of(q);
          if (!mbar_wait_ns(ready_bar(st), use_parity(q), P.wait_ns)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          if (ks == 0) mbar_arrive(exp_bar(it % kOgExpSlots));  // this item's row exponents are written
          const uint32_t ta = tmem + kOgAccCols + st * kOgStageCols;
          // B of pair pp: 16 - 2pp rows into the slot's tile (the descriptor
          // address field counts 16-byte units)
          const uint64_t dbs = db0 + (uint64_t)(xslot_of(q) * (kOgXBytes / 16));
#pragma unroll
          for (int pp = 0; pp < kOgPairs; ++pp)
            mma_f16kind_ta(tmem + (uint32_t)(tb * 32), ta + pp * kOgTileCols, dbs - (uint64_t)(2 * pp), kOgIdesc,
                           (ks | pp) ? 1u : 0u);
          any_mma = true;
          mma_commit(free_bar(st));
          mma_commit(bempty_bar(xslot_of(q)));
        }
        if (!ok) break;
        if (!(P.withhold && it == 0)) mma_commit(tfull_bar(tb));
      }
      if (!ok) atomicExch(P.err, 1);
      // after a timeout, or with a withheld commit (nobody else then waits
      // for the last MMAs), the MMAs in flight complete before the tensor
      // memory is freed
      if ((!ok || P.withhold) && any_mma) {
        mma_commit(drain_bar);
        mbar_wait(drain_bar, 0);
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
    const int chunks = (int)P.nchunks;
    int64_t tile = w0 / P.nchunks;
    int c = (int)(w0 % P.nchunks) - 1;
    for (int64_t w = w0; w < w1 && ok; ++w, ++it) {
      if (++c == chunks) {
        c = 0;
        ++tile;
      }
      if (tile != cur) {
        if (cur >= 0) flush(cur);
        wacc_init(acc);
        gmax = kOgNoGmax;
        nch = spec = 0;
        cur = tile;
      }
      const int F = __ldg(P.xexp + c);  // read early: its latency overlaps the waits
      const int tb = it % kOgAccBufs;
      if (!mbar_wait_ns(exp_bar(it % kOgExpSlots), (it / kOgExpSlots) & 1u, P.wait_ns)) {
        ok = false;
        break;
      }
      const int ev = exps[(it % kOgExpSlots) * kOgRows + rit];
      if (!mbar_wait_ns(tfull_bar(tb), (it / kOgAccBufs) & 1u, P.wait_ns)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      int32_t D[kOgDiags];
      {
        uint32_t rr[kOgDiags];
        tmem_ld20(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(tb * 32), rr);
#pragma unroll
        for (int g = 0; g < kOgDiags; ++g) D[g] = __float2int_rn(__uint_as_float(rr[g]));
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(tempty_bar(tb));
      const int E = ev >> 1;
      spec |= (uint32_t)ev & 1u;
      if (F == kOgXSpecial) {
        spec = 1;
      } else if (F != kOgNoExp) {
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
__global__ void __launch_bounds__(64)
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
  L.xexp = L.xdig + og_round256((size_t)L.nchunks * kOgKSteps * kOgXBytes);
  L.err = L.xexp + og_round256((size_t)L.nchunks * 4);
  L.part = L.err + 256;
  L.total = L.part + og_round256((size_t)L.tiles * L.segs * kOgRows * sizeof(OgPartial));
  return L;
}

// Test hook of quadblas_debug_stall_next_call (Ozaki qgemv).
static std::atomic<int> g_stall_qgemv{0};
void ozgemv_debug_stall_next() { g_stall_qgemv.store(1); }

size_t gemv_ozaki_scratch_bytes(int64_t m, int64_t n) {
  if (m <= 0 || n <= 0) return 0;
  return og_layout(m, n).total;
}

cudaError_t launch_gemv_ozaki(int64_t m, int64_t n, q128 alpha, MatView A, const q128* x, int64_t incx,
                              q128 beta, q128* y, int64_t incy, RowList* list, void* scratch, cudaStream_t s) {
  const bool row_major = A.sj == 1;
  const int64_t ld = row_major ? A.si : A.sj;
  if (!row_major && A.si != 1) return cudaErrorInvalidValue;
  // column-major A as (8 rows, row groups, columns) when m is a multiple of 8
  // (a box never reaches past the last row), else as 2-D (rows, columns)
  const int layout = row_major ? kOgRowMajor : (m % 8 == 0 ? kOgColGroups : kOgColBoxes);
  CUtensorMap map;
  {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return cudaErrorNotSupported;
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult rc;
    if (layout == kOgColGroups) {
      cuuint64_t dims[3] = {32, (cuuint64_t)(m / 8), (cuuint64_t)n};
      cuuint64_t strides[2] = {128, (cuuint64_t)ld * 16};
      cuuint32_t box[3] = {32, kOgRows / 8, (cuuint32_t)kOgKStep};
      rc = fn(&map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, const_cast<q128*>(A.p), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    } else {
      // A as 32-bit words, [rows][4 * cols] (row-major) or [cols][4 * rows]
      const int64_t inner = row_major ? n : m, outer = row_major ? m : n;
      cuuint64_t dims[2] = {(cuuint64_t)(4 * inner), (cuuint64_t)outer};
      cuuint64_t strides[1] = {(cuuint64_t)ld * 16};
      cuuint32_t box[2] = {32, row_major ? (cuuint32_t)kOgRows : (cuuint32_t)kOgKStep};  // 128 B x rows / columns
      rc = fn(&map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, const_cast<q128*>(A.p), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    }
    if (rc != CUDA_SUCCESS) return cudaErrorInvalidValue;
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
  const bool stall = g_stall_qgemv.exchange(0) != 0;  // test hook: this call's kernel times out
  P.wait_ns = stall ? kStallWaitNs : kWaitLimitNs;
  P.withhold = stall ? 1 : 0;
  cudaError_t e = cudaMemsetAsync(P.err, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  og_x_split_kernel<<<(unsigned)Lo.nchunks, 32, 0, s>>>(n, Lo.nchunks, x, incx, const_cast<uint8_t*>(P.xdig),
                                                        const_cast<int32_t*>(P.xexp), list);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  // the attribute is per device (and per host thread race-free)
  static std::atomic<bool> attr_set[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (!attr_set[dev].load(std::memory_order_acquire)) {
    if ((e = cudaFuncSetAttribute(og_gemv_kernel<kOgRowMajor>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kOgSmem)) != cudaSuccess ||
        (e = cudaFuncSetAttribute(og_gemv_kernel<kOgColGroups>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kOgSmem)) != cudaSuccess ||
        (e = cudaFuncSetAttribute(og_gemv_kernel<kOgColBoxes>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kOgSmem)) != cudaSuccess)
      return e;
    attr_set[dev].store(true, std::memory_order_release);
  }
  if (layout == kOgRowMajor)
    og_gemv_kernel<kOgRowMajor><<<(unsigned)Lo.G, kOgThreads, kOgSmem, s>>>(map, P);
  else if (layout == kOgColGroups)
    og_gemv_kernel<kOgColGroups><<<(unsigned)Lo.G, kOgThreads, kOgSmem, s>>>(map, P);
  else
    og_gemv_kernel<kOgColBoxes><<<(unsigned)Lo.G, kOgThreads, kOgSmem, s>>>(map, P);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  og_finish_kernel<<<(unsigned)((m + 63) / 64), 64, 0, s>>>(m, Lo.nchunks, Lo.work, Lo.G, Lo.segs, P.part,
                                                              P.err, alpha, beta, y, incy, list);
  return cudaGetLastError();
}

}  // namespace qb
