// Ozaki-split qgemm on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// Replaces the reference's soft-float GEMM loops
// (include/quadblas/algorithms/level3.hpp:17-336) by an error-free integer
// splitting (ozaki.cuh): each row of op(A) and column of op(B) is cut into s
// balanced digits of b bits (b = 9: stored as fp16; b = 8 or 7: as bf16),
// every digit pair (t, u) with t + u < s is an exact 16-bit-float ->
// fp32 GEMM on tcgen05.mma kind::f16 (integer sums below 2^24 stay exact,
// so k is read out of tensor memory in chunks of 256, 1024 or 4096), the
// pairs of one diagonal g = t + u are summed exactly in int32 (in k passes
// when a pass would overflow), and a fold kernel combines the diagonals into
// a 192-bit integer per output that is rounded once to binary128 and passed
// through the reference epilogue C = fma(alpha, sum, beta * C)
// (level3.hpp:107).
//
// tcgen05 kind::i8 does not exist on sm_103a, so integer digits travel as
// 16-bit floats: bf16 holds every integer up to 256 exactly, fp16 up to 2048.
//
// The default scheme is the residue (CRT) form of the same splitting
// (ozcrt.cuh): the truncated integers are reduced modulo N coprime moduli
// p_q in (256, 513], one exact residue GEMM per modulus, and the integer
// result is rebuilt by the Chinese remainder theorem before the rounding.
//
// Kernels:
//   ozaki_init_kernel,  : starting values of the scales and flags (and, on
//   ozaki_fill_kernel     one stream, the error words)
//   ozaki_scale_kernel,   : S_i = max_l (exponent(x_il) + 1) per row of a
//   ozaki_scale_rows_kernel strided view (A, or B^T), plus NaN/inf flags
//   ozaki_split_kernel  : digits of every element, written digit-major and
//                         K-major: D[t][row][l], zero padded
//   ozaki_crt_split_tc_kernel: residues of every element on the tensor cores
//                         (byte rows of the scaled integer times a table of
//                         256^j mod p_q), one fp32 remainder per residue
//                         (two elements per packed fp32 instruction); for
//                         op(B) on one stream, a fifth warp takes op(A)'s
//                         row scales meanwhile
//   ozaki_mma_kernel    : persistent, warp-specialised: warp 0 issues TMA
//                         loads (128B-swizzled 64-wide K slices of A_t and
//                         B_u) into a 4-stage shared-memory ring, warp 1
//                         issues tcgen05.mma (M=128, N=256, K=16) into one
//                         of two 256-column fp32 accumulators in tensor
//                         memory, warps 2..9 read the accumulators with
//                         tcgen05.ld and store a diagonal's int32 sum
//                         (digit pairs) or a modulus's u16 residue (CRT).
//                         With two or more tile rows, CTAs run in clusters
//                         of two over vertically adjacent tiles and each
//                         loads half of the shared B slice, multicast to
//                         both.  Every mbarrier wait is bounded (1 s); on
//                         timeout the kernel records an error, drains its
//                         own copies and MMAs, frees tensor memory and exits.
//   ozaki_fold_kernel   : Horner fold of C_0..C_G (and k passes) per output,
//                         one rounding, reference epilogue
//   ozaki_crt_pass_sum_kernel, ozaki_crt_fold_tc_kernel: the residues of k
//                         passes summed mod p_q; the CRT reconstruction with
//                         its word sums on the tensor cores (y_q times the
//                         bytes of M / p_q), one rounding, reference epilogue
//   ozaki_special_kernel: outputs whose row or column holds NaN or inf, by a
//                         direct wide-accumulator dot, so specials keep IEEE
//                         semantics (returns at once when there are none)
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <stdio.h>
#include <stdlib.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <vector>

#include "kernels.h"
#include "ozaki.cuh"
#include "ozcrt.cuh"
#include "reduce.cuh"
#include "umma.cuh"

namespace qb {

// ---------------------------------------------------------------------------
// Scaling and splitting
// ---------------------------------------------------------------------------
// One thread per (row, chunk of 64 columns) of the view X(r, c) = p[r*sr + c*sc];
// *any is set when a NaN or infinity is seen.
__global__ void ozaki_scale_kernel(int64_t rows, int64_t cols, const q128* __restrict__ p,
                                   int64_t sr, int64_t sc, int* __restrict__ S,
                                   uint32_t* __restrict__ flags, int* __restrict__ any) {
  pdl_wait();
  pdl_trigger();
  const int64_t nchunk = (cols + 63) / 64;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < rows * nchunk; w += stride) {
    int64_t r, ch;
    if (sr == 1) {  // rows contiguous in memory: consecutive threads take consecutive rows
      r = w % rows;
      ch = w / rows;
    } else {
      r = w / nchunk;
      ch = w % nchunk;
    }
    int64_t c0 = ch * 64, c1 = c0 + 64 < cols ? c0 + 64 : cols;
    int mx = kOzakiScaleEmpty;
    uint32_t fl = 0;
    for (int64_t c = c0; c < c1; ++c) {
      q128 v = ld_cached(p + r * sr + c * sc);
      int e = ozaki_exp_plus1(v);
      mx = e > mx ? e : mx;
      fl |= ozaki_special_flags(v);
    }
    if (mx != kOzakiScaleEmpty) atomicMax(S + r, mx);
    if (fl) {
      atomicOr(flags + r, fl);
      atomicOr(any, 1);
    }
  }
}

// The same for views whose columns are contiguous (sc = 1): one warp per
// (row, chunk of 256 columns), each lane reading every 32nd element, so that
// a warp's loads cover 512 contiguous bytes; warp maximum by shuffles.
__global__ void __launch_bounds__(256)
    ozaki_scale_rows_kernel(int64_t rows, int64_t cols, const q128* __restrict__ p, int64_t sr,
                            int* __restrict__ S, uint32_t* __restrict__ flags, int* __restrict__ any) {
  pdl_wait();
  pdl_trigger();
  const int lane = threadIdx.x & 31;
  const int64_t nchunk = (cols + 255) / 256;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x / 32);
  for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32; w < rows * nchunk; w += nwarps) {
    const int64_t r = w / nchunk, c0 = (w % nchunk) * 256;
    const q128* row = p + r * sr;
    int mx = kOzakiScaleEmpty;
    uint32_t fl = 0;
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const int64_t c = c0 + lane + 32 * t;
      if (c < cols) {
        const q128 v = ld_stream(row + c);
        mx = max(mx, ozaki_exp_plus1(v));
        fl |= ozaki_special_flags(v);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mx = max(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, o));
      fl |= __shfl_xor_sync(0xFFFFFFFFu, fl, o);
    }
    if (lane == 0) {
      if (mx != kOzakiScaleEmpty) atomicMax(S + r, mx);
      if (fl) {
        atomicOr(flags + r, fl);
        atomicOr(any, 1);
      }
    }
  }
}

// Launches kern on st; with pdl, as a programmatic dependent of the kernel
// before it in the stream (its launch may start while that kernel runs;
// the kernel's pdl_wait orders its memory accesses after it).
template <typename... KArgs, typename... Args>
static cudaError_t launch_maybe_pdl(bool pdl, void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem,
                                    cudaStream_t st, Args... args) {
  if (!pdl) {
    kern<<<grid, block, smem, st>>>(args...);
    return cudaGetLastError();
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, args...);
}

// Scales and flags of a view (rows x cols), on stream st (pdl: as a
// programmatic dependent of the kernel before it).
static cudaError_t launch_scale(int64_t rows, int64_t cols, const q128* p, int64_t sr, int64_t sc, int* S,
                                uint32_t* flags, int* any, int sms, cudaStream_t st, bool pdl = false) {
  if (rows <= 0) return cudaSuccess;
  if (sc == 1) {
    const int64_t warps = rows * ((cols + 255) / 256);
    const unsigned b = (unsigned)std::max<int64_t>(1, std::min<int64_t>((warps + 7) / 8, (int64_t)sms * 8));
    return launch_maybe_pdl(pdl, ozaki_scale_rows_kernel, dim3(b), dim3(256), 0, st, rows, cols, p, sr, S, flags,
                            any);
  }
  const int64_t w = rows * ((cols + 63) / 64);
  const unsigned b = (unsigned)std::max<int64_t>(1, std::min<int64_t>((w + 255) / 256, (int64_t)sms * 8));
  return launch_maybe_pdl(pdl, ozaki_scale_kernel, dim3(b), dim3(256), 0, st, rows, cols, p, sr, sc, S, flags, any);
}

// One-stream form of the two fills and the error-word resets: S, fa for m
// rows, F, fb for n, and err[0], [1], [2], [4], [5] zeroed.
__global__ void ozaki_init_kernel(int64_t m, int* __restrict__ S, uint32_t* __restrict__ fa, int64_t n,
                                  int* __restrict__ F, uint32_t* __restrict__ fb, int* __restrict__ err) {
  pdl_wait();
  pdl_trigger();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) {
    S[i] = kOzakiScaleEmpty;
    fa[i] = 0u;
  }
  if (i < n) {
    F[i] = kOzakiScaleEmpty;
    fb[i] = 0u;
  }
  if (i == 0) err[0] = err[1] = err[2] = err[4] = err[5] = 0;
}

__global__ void ozaki_fill_kernel(int64_t n, int* __restrict__ S, uint32_t* __restrict__ flags) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    S[i] = kOzakiScaleEmpty;
    flags[i] = 0u;
  }
}

// Digits of the (rows_pad x cols_pad) zero-padded view: digit t of element
// (r, c) goes to D[t * plane + r * cols_pad + c]; rows in [rows, rows_pad)
// and columns in [cols, cols_pad) get zero digits.  Block (32, 8): x along
// columns (coalesced digit stores), y along rows.  A thread cuts two
// neighbouring columns (c, c+1) of a row and stores each digit pair as one
// 32-bit word (cols_pad is a multiple of 64, so c is even); each digit is
// stored as soon as it is extracted.
// Digits are stored as bf16 (b = 7, 8) or fp16 (b = 9), two per 32-bit word.
template <int B>
__device__ __forceinline__ uint32_t pack_digits(int d0, int d1) {
  if (B == 9) {
    __half2 h = __floats2half2_rn((float)d0, (float)d1);
    return *reinterpret_cast<uint32_t*>(&h);
  } else {
    __nv_bfloat162 h = __floats2bfloat162_rn((float)d0, (float)d1);
    return *reinterpret_cast<uint32_t*>(&h);
  }
}

template <int B>
__global__ void __launch_bounds__(256)
    ozaki_split_kernel(int64_t rows, int64_t cols, int64_t rows_pad, int64_t cols_pad, int64_t plane,
                       const q128* __restrict__ p, int64_t sr, int64_t sc,
                       const int* __restrict__ S, int s, uint16_t* __restrict__ D) {
  const int64_t c = ((int64_t)blockIdx.x * 32 + threadIdx.x) * 2;
  const int64_t r = (int64_t)blockIdx.y * 8 + threadIdx.y;
  if (c >= cols_pad || r >= rows_pad) return;
  const int64_t plane2 = plane / 2;
  uint32_t* out = reinterpret_cast<uint32_t*>(D + r * cols_pad + c);
  q128 v0 = q_zero(0), v1 = q_zero(0);
  int Sr = kOzakiScaleEmpty;
  if (r < rows) {
    Sr = S[r];
    if (c < cols) v0 = ld_cached(p + r * sr + c * sc);
    if (c + 1 < cols) v1 = ld_cached(p + r * sr + (c + 1) * sc);
  }
  ozaki_digits_emit2<B>(v0, v1, Sr, s, [&](int t, int d0, int d1) { out[t * plane2] = pack_digits<B>(d0, d1); });
}

// Residues for the CRT scheme on the tensor cores (ozcrt.cuh, "Residue split
// on the tensor cores"): residue q of element (r, c) of the same view goes to
// D[q * plane + r * cols_pad + c] as fp16, rows in [rows, rows_pad) and
// columns in [cols, cols_pad) as zeros.  Persistent CTAs of 4 warps walk
// tiles of 4 rows x 64 columns: warp w takes row 4t + w, lane l columns 2l
// and 2l + 1 (one tensor-memory lane, two elements).  Per tile each thread
// scales its two elements (crt_scaled_words, branch-free), writes their
// operand rows (32 fp16 each: s (1024 + b_j), -s, zeros) to tensor memory;
// one thread issues four MMAs (M = 128, K = 16, N = 2 NP, block-diagonal B:
// element e of modulus q in column 2q + e) against the table in shared
// memory and waits for them; then each thread reads its x_q, rounds
// r = x - p round(x / p) in fp32 (exact, |r| <= 256) and stores the two
// residues of a modulus as one 32-bit word.  The next tile's elements are
// loaded while the MMAs run.  128 tensor-memory columns per CTA (D: [0, 96),
// A: [96, 128)), four CTAs per SM.  The wait for the MMAs is bounded (1 s);
// on a timeout the CTA stops, records it in *err and frees its tensor memory.
// Optionally a fifth warp per CTA computes, meanwhile, the row scales and
// flags of the other operand (rows contiguous, as ozaki_scale_rows_kernel
// does, one warp per whole row): that operand's own scale launch then goes,
// and its reads use the bandwidth the split leaves.  The four split warps
// synchronise among themselves (named barrier 1).
struct CrtSplitParams {
  int64_t rows, cols, rows_pad, cols_pad, plane;
  const q128* p;
  int64_t sr, sc;
  const int* S;
  int* err;
  uint16_t* D;
  // side job (xs_p null: none): rows [0, xs_rows) of xs_p, row r at
  // xs_p + r * xs_sr, xs_cols contiguous elements; S and flags of each row
  // are stored (the row is this warp's alone), *xs_any set on NaN or inf
  const q128* xs_p;
  int64_t xs_rows, xs_cols, xs_sr;
  int* xs_S;
  uint32_t* xs_flags;
  int* xs_any;
};

constexpr int kSplitThreads = 128;
constexpr int kSplitSideThreads = kSplitThreads + 32;  // with the side job's warp
constexpr int kSplitTmemCols = 128;
constexpr int kSplitAcol = 96;
constexpr int kSplitCtasPerSm = 4;
constexpr size_t kSplitSmem = 48 * 1024;  // table + barrier; also keeps a fifth CTA off the SM

// Operand row of one element: bytes 2i, 2i+1 of V as fp16 s (1024 + b),
// then -s, then zeros.
template <int NB>
__device__ __forceinline__ void crt_operand_row(q128 v, int Sr, int T, uint32_t* a) {
  constexpr int NW = (NB + 3) / 4;
  uint32_t w[NW];
  bool neg;
  crt_scaled_words<NW>(v, Sr, T, w, neg);
  const uint32_t sgn = neg ? 0xE4E4E4E4u : 0x64646464u;
#pragma unroll
  for (int i = 0; i < NB / 2; ++i) a[i] = __byte_perm(w[i >> 1], sgn, (i & 1) ? 0x4342u : 0x4140u);
  a[NB / 2] = neg ? 0x3C00u : 0xBC00u;
#pragma unroll
  for (int i = NB / 2 + 1; i < 16; ++i) a[i] = 0u;
}

// The side job's rows [r0, r1): per row the largest exponent(x) + 1 and the
// special-value flags, 8 loads of 16 bytes per lane in flight (a warp reads
// 4 KiB of the row at a time).
__device__ __forceinline__ void split_side_row_scales(const CrtSplitParams& P, int64_t r0, int64_t r1, int lane) {
  for (int64_t r = r0; r < r1; ++r) {
    const q128* row = P.xs_p + r * P.xs_sr;
    int mx = kOzakiScaleEmpty;
    uint32_t fl = 0;
    for (int64_t c0 = 0; c0 < P.xs_cols; c0 += 256) {
      q128 v[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const int64_t c = c0 + lane + 32 * t;
        v[t] = c < P.xs_cols ? ld_stream(row + c) : q_zero(0);
      }
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        mx = max(mx, ozaki_exp_plus1(v[t]));
        fl |= ozaki_special_flags(v[t]);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mx = max(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, o));
      fl |= __shfl_xor_sync(0xFFFFFFFFu, fl, o);
    }
    if (lane == 0) {
      P.xs_S[r] = mx;
      P.xs_flags[r] = fl;
      if (fl) atomicOr(P.xs_any, 1);
    }
  }
}

__device__ __forceinline__ void split_warps_sync() { asm volatile("bar.sync 1, 128;" ::: "memory"); }

template <int NB>
__global__ void __launch_bounds__(kSplitSideThreads)
    ozaki_crt_split_tc_kernel(const __grid_constant__ CrtSplitParams P, const __grid_constant__ CrtSplitTable tab) {
  extern __shared__ __align__(128) uint8_t split_smem[];
  uint8_t* sbase = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(split_smem) + 127) & ~(uintptr_t)127);
  uint64_t* bar = reinterpret_cast<uint64_t*>(sbase + kCrtSplitK * kCrtSplitMaxN * 2);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 1);
  int* flag = reinterpret_cast<int*>(bar + 2);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int N = tab.N, nmod = tab.nmod;
  // the table (B operand) into shared memory, visible to the tensor cores
  for (int i = threadIdx.x; i < N * kCrtSplitK / 8 && warp < 4; i += kSplitThreads)
    reinterpret_cast<uint4*>(sbase)[i] = reinterpret_cast<const uint4*>(tab.b)[i];
  fence_proxy_async_smem();
  if (threadIdx.x == 0) {
    mbar_init(smem_u32(bar), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kSplitTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  pdl_wait();
  pdl_trigger();
  const uint32_t tlane = tmem + ((uint32_t)(warp * 32) << 16);
  const uint32_t idesc = (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
  const uint32_t sb = smem_u32(sbase), lbo = (uint32_t)N * 16u;
  const int64_t plane2 = P.plane / 2;

  // tiles t = blockIdx.x, + gridDim.x, ...: (row tile tr, column tile tc),
  // advanced by counting (no division in the loop)
  const int tiles_c = (int)(P.cols_pad / 64), tiles_r = (int)(P.rows_pad / 4);
  const int step_r = (int)gridDim.x / tiles_c, step_c = (int)gridDim.x % tiles_c;
  int tr = (int)blockIdx.x / tiles_c, tc = (int)blockIdx.x % tiles_c;
  auto load = [&](int r_t, int c_t, q128& v0, q128& v1, int& Sr) {
    v0 = v1 = q_zero(0);
    Sr = kOzakiScaleEmpty;
    if (r_t >= tiles_r) return;
    const int64_t r = (int64_t)r_t * 4 + warp, c = (int64_t)c_t * 64 + 2 * lane;
    if (r < P.rows) {
      Sr = P.S[r];
      const q128* e = P.p + r * P.sr + c * P.sc;
      if (c < P.cols) v0 = ld_cached(e);
      if (c + 1 < P.cols) v1 = ld_cached(e + P.sc);
    }
  };
  if (warp == 4) {
    // the side job (launched with it only); this warp takes no tiles
    const int64_t G = gridDim.x;
    split_side_row_scales(P, P.xs_rows * blockIdx.x / G, P.xs_rows * (blockIdx.x + 1) / G, lane);
    tr = tiles_r;
  }
  // elements of this tile (v0, v1, Sr), the next (n*) and the one after it,
  // loaded while the MMAs of this tile run: two tiles in flight
  q128 v0, v1, n0, n1;
  int Sr, nS;
  load(tr, tc, v0, v1, Sr);
  int fr = tr, fc = tc;  // the tile whose elements were loaded last
  auto advance = [&](int& r_t, int& c_t) {
    c_t += step_c;
    r_t += step_r;
    if (c_t >= tiles_c) {
      c_t -= tiles_c;
      ++r_t;
    }
  };
  advance(fr, fc);
  load(fr, fc, n0, n1, nS);
  uint32_t phase = 0;
  bool ok = true;
  while (tr < tiles_r) {
    {
      uint32_t a[32];
      crt_operand_row<NB>(v0, Sr, tab.T, a);
      crt_operand_row<NB>(v1, Sr, tab.T, a + 16);
      tmem_st32(tlane + kSplitAcol, a);
    }
    tmem_st_wait();
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    split_warps_sync();  // operand rows written; the last tile's accumulator read
    const int64_t r = (int64_t)tr * 4 + warp, c = (int64_t)tc * 64 + 2 * lane;
    advance(tr, tc);
    if (threadIdx.x == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int kt = 0; kt < 4; ++kt)
        mma_f16kind_ta(tmem, tmem + kSplitAcol + 8 * kt, smem_desc_noswizzle(sb + 2 * kt * lbo, lbo, 128), idesc,
                       kt ? 1u : 0u);
      mma_commit(smem_u32(bar));
    }
    v0 = n0;
    v1 = n1;
    Sr = nS;
    advance(fr, fc);
    load(fr, fc, n0, n1, nS);  // two tiles ahead, in flight while the MMAs run
    if (threadIdx.x == 0) *flag = mbar_wait(smem_u32(bar), phase) ? 1 : 0;
    phase ^= 1u;
    split_warps_sync();
    if (!*flag) {
      ok = false;
      break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    uint32_t* out = reinterpret_cast<uint32_t*>(P.D + r * P.cols_pad + c);
    // groups of 8 moduli (16 columns), unrolled so that every modulus index is
    // a constant and its p and 1/p come straight from the parameter bank
#pragma unroll
    for (int g = 0; g < kCrtMaxMods / 8; ++g) {
      if (8 * g < nmod) {
        uint32_t x[16];
        tmem_ld16(tlane + 16 * g, x);
        const bool whole = 8 * g + 8 <= nmod;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int q = 8 * g + i;
          if (whole || q < nmod) {
            // both elements at once: u = round(x / p) (x fl(1/p) + 1.5 2^23,
            // then - 1.5 2^23), r = x - u p
            constexpr uint64_t kMagic = 0x4B4000004B400000ull, kNegMagic = 0xCB400000CB400000ull;
            const uint64_t xx = f32x2_pack(x[2 * i], x[2 * i + 1]);
            const uint64_t uu = f32x2_add(f32x2_fma(xx, tab.inv_p2[q], kMagic), kNegMagic);
            uint32_t r0, r1;
            f32x2_unpack(f32x2_fma(uu, tab.neg_p2[q], xx), r0, r1);
            const __half2 h = __floats2half2_rn(__uint_as_float(r0), __uint_as_float(r1));
            out[q * plane2] = *reinterpret_cast<const uint32_t*>(&h);
          }
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  }
  if (!ok && threadIdx.x == 0) atomicExch(P.err, 1);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kSplitTmemCols)
                 : "memory");
}

// ---------------------------------------------------------------------------
// tcgen05 digit GEMM
// ---------------------------------------------------------------------------
constexpr int kBM = 128, kBN = 256, kBK = 64;  // tile; kBK 16-bit digits = 128 bytes per row
constexpr int kStages = 4;
constexpr int kStageA = kBM * kBK * 2;          // 16 KiB
constexpr int kStageB = kBN * kBK * 2;          // 32 KiB
constexpr int kStageBytes = kStageA + kStageB;  // 48 KiB
constexpr int kMmaThreads = 320;                // 10 warps
constexpr int kEpiWarps = 8;
constexpr int kTmemCols = 512;                  // two 256-column fp32 accumulators
constexpr size_t kMmaSmem = (size_t)kStages * kStageBytes + 1024 + 256;

struct OzakiMmaParams {
  int tiles_m, tiles_n;
  int tile_begin, tile_end;  // tiles of this launch (tile = tm * tiles_n + tn)
  uint32_t idesc;            // instruction descriptor (bf16 or fp16 digits)
  int G;                     // highest diagonal (s - 1)
  int m_pad, n_pad;          // shape of the output planes (C or Y)
  int pa, pb;                // rows of one digit / residue plane of A and of B
  // grouped problems: tile v of the launch multiplies A tile list[v].a_tile
  // by B tile list[v].b_tile and stores output tile (v, 0); null otherwise
  const OzakiGroupTile* list;
  int kb_begin, kb_end;  // k-blocks of this pass
  int chunk_kb;          // k-blocks summed exactly in fp32 before a readout
  int32_t* C;            // [G+1][m_pad][n_pad] (digit pairs)
  int* err;              // set to nonzero on a timeout
  // CRT scheme: unit g is the single pair (g, g), the residue product of
  // modulus g, and the epilogue stores y = (C mod p) u mod p (16 bits) in Y
  int crt;
  uint16_t* Y;                  // [G+1][m_pad][n_pad], fp16 values
  uint32_t crt_p[kCrtMaxMods], crt_magic[kCrtMaxMods], crt_K[kCrtMaxMods], crt_u[kCrtMaxMods];
  // Paired CTAs (launched as clusters of two): the two CTAs of a cluster
  // take tile rows 2r and 2r + 1 of the same tile column in lockstep, each
  // loads its A tile and one half (128 rows) of the shared B tile with a
  // multicast copy to both, and a stage is refilled once both CTAs' MMAs
  // released it.  tile_begin and tile_end are then whole tile rows.
  int pair;
  // test hook (quadblas_debug_stall_next_call): pipeline waits give up after
  // wait_ns; withhold = 1 makes the MMA issuer skip the accumulator-full
  // commit of its first chunk, so that the epilogue's wait runs out
  unsigned long long wait_ns;
  int withhold;
};

// Instruction descriptors: kind::f16, D = f32, K-major A and B, N = 256,
// M = 128; A and B both bf16 (bits 7-9 and 10-12 = 1) or both fp16 (= 0).
constexpr uint32_t kIdescShape = (1u << 4) | ((uint32_t)(kBN >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);
constexpr uint32_t kIdescBf16 = kIdescShape | (1u << 7) | (1u << 10);
constexpr uint32_t kIdescF16 = kIdescShape;

// The (tile, diagonal) units of one CTA, in order.  Digit pairs: tiles come
// in full waves of gridDim.x: CTA c takes tile w * gridDim.x + c and runs all
// its diagonals, highest first, so every CTA of a wave issues the same
// sequence of (diagonal, pair, k block) loads at the same time and the digit
// panels they share (A_t of a tile row, B_u of a tile column) are read from
// DRAM once per wave rather than once per CTA.  The tiles left over after the
// full waves are spread as (tile, diagonal) units, highest diagonal first.
// Residues: each modulus's planes are used by one unit per tile and by no
// other modulus, so units are dealt modulus-major (unit v = c + j gridDim.x
// is modulus G - v / tiles of tile v % tiles): all tiles of a modulus run
// before the next modulus starts, and its two planes (2 x 32 MB at 4096^2)
// stay in L2 across the waves instead of being streamed again per wave.
//
// A CTA's place in the deal: its index and the count among the dealers (the
// cluster index and count for paired CTAs), and the tiles dealt (tile-row
// pairs x tile columns for paired CTAs).
struct UnitDeal {
  int c, G, tiles, rank;
};

__device__ __forceinline__ UnitDeal unit_deal(const OzakiMmaParams& P) {
  UnitDeal d;
  const int tiles = P.tile_end - P.tile_begin;
  if (P.pair) {
    d.rank = (int)cluster_ctarank();
    d.c = (int)blockIdx.x >> 1;
    d.G = (int)gridDim.x >> 1;
    d.tiles = (tiles / P.tiles_n + 1) / 2 * P.tiles_n;
  } else {
    d.rank = 0;
    d.c = (int)blockIdx.x;
    d.G = (int)gridDim.x;
    d.tiles = tiles;
  }
  return d;
}

__device__ __forceinline__ int cta_unit_count(const OzakiMmaParams& P, const UnitDeal& d) {
  const int tiles = d.tiles, G1 = P.G + 1;
  if (P.crt) {
    const int left = tiles * G1 - d.c;
    return left > 0 ? (left + d.G - 1) / d.G : 0;
  }
  const int waves = tiles / d.G, rem = tiles - waves * d.G;
  const int tail = rem * G1 - d.c;
  return waves * G1 + (tail > 0 ? (tail + d.G - 1) / d.G : 0);
}

// Unit j of this CTA: its operand tiles (tm of A, tn of B), output tile
// (ym, yn), diagonal or modulus g, and whether the tile exists (the second
// CTA of a pair past an odd last tile row computes a tile of its own that is
// not stored).
__device__ __forceinline__ void cta_unit(const OzakiMmaParams& P, const UnitDeal& d, int j, int& tm, int& tn,
                                         int& ym, int& yn, int& g, bool& real) {
  const int tiles = d.tiles, G1 = P.G + 1;
  int vt;
  if (P.crt) {
    const int v = d.c + j * d.G;
    g = P.G - v / tiles;
    vt = v % tiles;
  } else {
    const int waves = tiles / d.G, rem = tiles - waves * d.G;
    if (j < waves * G1) {
      vt = (j / G1) * d.G + d.c;
      g = P.G - j % G1;
    } else {
      const int v = d.c + (j - waves * G1) * d.G;
      g = P.G - v / rem;
      vt = waves * d.G + v % rem;
    }
  }
  if (!P.pair) {
    const int tile = P.tile_begin + vt;
    if (P.list) {
      tm = P.list[tile].a_tile;
      tn = P.list[tile].b_tile;
      ym = tile;
      yn = 0;
    } else {
      tm = ym = tile / P.tiles_n;
      tn = yn = tile % P.tiles_n;
    }
    real = true;
    return;
  }
  const int row0 = P.tile_begin / P.tiles_n, rows = (P.tile_end - P.tile_begin) / P.tiles_n;
  const int r = 2 * (vt / P.tiles_n) + d.rank;
  tn = yn = vt % P.tiles_n;
  tm = ym = row0 + r;
  real = r < rows;
}

__global__ void __launch_bounds__(kMmaThreads, 1)
    ozaki_mma_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                     const __grid_constant__ CUtensorMap tmBh, OzakiMmaParams P) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;  // 128B swizzle needs 1024-byte alignment
  uint8_t* gbase = smem_raw + (base - raw);
  // barriers and the tensor-memory address live after the stages
  const uint32_t bar0 = base + kStages * kStageBytes;
  auto full_bar = [&](int s) { return bar0 + 8u * s; };
  auto empty_bar = [&](int s) { return bar0 + 8u * (kStages + s); };
  auto tfull_bar = [&](int b) { return bar0 + 8u * (2 * kStages + b); };
  auto tempty_bar = [&](int b) { return bar0 + 8u * (2 * kStages + 2 + b); };
  const uint32_t drain_bar = bar0 + 8u * (2 * kStages + 4);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(gbase + kStages * kStageBytes + 8 * (2 * kStages + 5));

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(full_bar(s), 1);
      mbar_init(empty_bar(s), P.pair ? 2 : 1);  // paired: both CTAs' MMAs release a stage
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(tfull_bar(b), 1);
      mbar_init(tempty_bar(b), kEpiWarps);
    }
    mbar_init(drain_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  // paired: the peer's barriers are initialised before any copy or commit reaches them
  if (P.pair) cluster_sync_all();
  pdl_wait();
  pdl_trigger();

  const UnitDeal deal = unit_deal(P);
  const int nun = cta_unit_count(P, deal);
  const int nkb = P.kb_end - P.kb_begin;
  const int nchunks = (nkb + P.chunk_kb - 1) / P.chunk_kb;
  bool ok = true;

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      uint32_t it = 0;
      for (int j = 0; j < nun && ok; ++j) {
        int tm, tn, ym, yn, g;
        bool real;
        cta_unit(P, deal, j, tm, tn, ym, yn, g, real);
        for (int t = P.crt ? g : 0; t <= g && ok; ++t) {
          const int u = P.crt ? g : g - t;
          for (int kb = P.kb_begin; kb < P.kb_end && ok; ++kb, ++it) {
            const int s = it % kStages;
            const uint32_t round = it / kStages;
            if (!mbar_wait_ns(empty_bar(s), (round & 1u) ^ 1u, P.wait_ns)) {
              ok = false;
              break;
            }
            mbar_expect_tx(full_bar(s), kStageBytes);
            const uint32_t sa = base + s * kStageBytes, sb = sa + kStageA;
            tma_load_2d(sa, &tmA, full_bar(s), kb * kBK, t * P.pa + tm * kBM);
            if (P.pair)  // this CTA's half of B, to both CTAs
              tma_load_2d_mc(sb + deal.rank * (kStageB / 2), &tmBh, full_bar(s), kb * kBK,
                             u * P.pb + tn * kBN + deal.rank * (kBN / 2), (uint16_t)3);
            else
              tma_load_2d(sb, &tmB, full_bar(s), kb * kBK, u * P.pb + tn * kBN);
          }
        }
      }
      if (!ok) {
        atomicExch(P.err, 1);
        // drain the copies still in flight: the last kStages issued fills
        for (uint32_t j = (it > kStages ? it - kStages : 0); j < it; ++j)
          mbar_wait(full_bar(j % kStages), (j / kStages) & 1u);
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      uint32_t it = 0, acc_it = 0;
      bool issued_any = false;
      for (int j = 0; j < nun && ok; ++j) {
        int tm, tn, ym, yn, g;
        bool real;
        cta_unit(P, deal, j, tm, tn, ym, yn, g, real);
        for (int t = P.crt ? g : 0; t <= g && ok; ++t) {
          for (int ch = 0; ch < nchunks && ok; ++ch) {
            const int kb0 = P.kb_begin + ch * P.chunk_kb;
            const int kb1 = kb0 + P.chunk_kb < P.kb_end ? kb0 + P.chunk_kb : P.kb_end;
            const int buf = acc_it & 1;
            const uint32_t round = acc_it >> 1;
            if (!mbar_wait_ns(tempty_bar(buf), (round & 1u) ^ 1u, P.wait_ns)) {
              ok = false;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t dcol = tmem + (uint32_t)(buf * kBN);
            for (int kb = kb0; kb < kb1; ++kb, ++it) {
              const int s = it % kStages;
              if (!mbar_wait_ns(full_bar(s), (it / kStages) & 1u, P.wait_ns)) {
                ok = false;
                break;
              }
              asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
              const uint32_t sa = base + s * kStageBytes, sb = sa + kStageA;
              const uint64_t da = smem_desc_sw128(sa), db = smem_desc_sw128(sb);
#pragma unroll
              for (int k = 0; k < kBK / 16; ++k) {
                // +32 bytes per K=16 step inside the 128-byte swizzled row
                mma_f16kind(dcol, da + (uint64_t)(2 * k), db + (uint64_t)(2 * k), P.idesc,
                            (kb > kb0 || k > 0) ? 1u : 0u);
              }
              issued_any = true;
              if (P.pair)
                mma_commit_mc(empty_bar(s), (uint16_t)3);  // the stage is free here and in the peer
              else
                mma_commit(empty_bar(s));
            }
            if (!ok) break;
            if (!(P.withhold && acc_it == 0)) mma_commit(tfull_bar(buf));
            ++acc_it;
          }
        }
      }
      if (!ok) atomicExch(P.err, 1);
      // after a timeout, or with a withheld commit (nobody else then waits
      // for the last MMAs), the MMAs in flight complete before the tensor
      // memory is freed
      if ((!ok || P.withhold) && issued_any) {
        mma_commit(drain_bar);
        mbar_wait(drain_bar, 0);
      }
    }
  } else {
    // ---------------- epilogue: 8 warps ----------------
    const int e = warp - 2;
    const int quad = warp & 3;           // tensor-memory lane quadrant of this warp
    const int half = e >> 2;             // column half: [0,128) or [128,256)
    const int row_in_tile = quad * 32 + lane;
    int32_t acc[kBN / 2];
#pragma unroll
    for (int i = 0; i < kBN / 2; ++i) acc[i] = 0;
    uint32_t acc_it = 0;
    for (int j = 0; j < nun && ok; ++j) {
      int tm, tn, ym, yn, g;
      bool real;
      cta_unit(P, deal, j, tm, tn, ym, yn, g, real);
      for (int t = P.crt ? g : 0; t <= g && ok; ++t) {
        for (int ch = 0; ch < nchunks && ok; ++ch) {
          const int buf = acc_it & 1;
          if (!mbar_wait_ns(tfull_bar(buf), (acc_it >> 1) & 1u, P.wait_ns)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t taddr =
              tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(buf * kBN + half * (kBN / 2));
          // 16 columns at a time, the next load in flight while these convert
          uint32_t ra[16], rb[16];
          tmem_ld16_nowait(taddr, ra);
#pragma unroll
          for (int c = 0; c < kBN / 2; c += 32) {
            tmem_ld_wait();
            tmem_ld16_nowait(taddr + (uint32_t)(c + 16), rb);
#pragma unroll
            for (int i = 0; i < 16; ++i) acc[c + i] += __float2int_rn(__uint_as_float(ra[i]));
            tmem_ld_wait();
            if (c + 32 < kBN / 2) tmem_ld16_nowait(taddr + (uint32_t)(c + 32), ra);
#pragma unroll
            for (int i = 0; i < 16; ++i) acc[c + 16 + i] += __float2int_rn(__uint_as_float(rb[i]));
          }
          tmem_ld_wait();
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          __syncwarp();
          if (lane == 0) mbar_arrive(tempty_bar(buf));
          ++acc_it;
        }
      }
      if (!ok) break;
      // store diagonal g of this tile: row (tm*128 + row_in_tile), 128 columns
      const size_t off = ((size_t)g * P.m_pad + (size_t)ym * kBM + row_in_tile) * P.n_pad + (size_t)yn * kBN +
                         half * (kBN / 2);
      // (a pair's second CTA past an odd last tile row computed a tile that
      // does not exist: nothing is stored)
      if (P.crt && real) {
        // |acc| <= 2^29 (a pass holds 8192 of k): y = ((acc mod p) u) mod p < 2^16
        const uint32_t p = P.crt_p[g], mg = P.crt_magic[g], K = P.crt_K[g], u = P.crt_u[g];
        uint16_t* dst = P.Y + off;
#pragma unroll
        for (int i = 0; i < kBN / 2; ++i)
          acc[i] = (int32_t)crt_mod(crt_mod((uint32_t)(acc[i] + (int32_t)K), p, mg) * u, p, mg);
        // stored as fp16 values (y <= 512 is exact): the bits 0x6400 + y are
        // 1024 + y, minus 1024 in pairs; the reconstruction multiplies them
        // on the tensor cores as they are
        auto h2 = [](int32_t y0, int32_t y1) {
          const uint32_t w = ((uint32_t)y0 | ((uint32_t)y1 << 16)) + 0x64006400u, k1024 = 0x64006400u;
          const __half2 v = __hsub2(*reinterpret_cast<const __half2*>(&w), *reinterpret_cast<const __half2*>(&k1024));
          return *reinterpret_cast<const uint32_t*>(&v);
        };
#pragma unroll
        for (int i = 0; i < kBN / 2; i += 8)
          *reinterpret_cast<uint4*>(dst + i) =
              make_uint4(h2(acc[i], acc[i + 1]), h2(acc[i + 2], acc[i + 3]), h2(acc[i + 4], acc[i + 5]),
                         h2(acc[i + 6], acc[i + 7]));
      } else if (real) {
        int32_t* dst = P.C + off;
#pragma unroll
        for (int i = 0; i < kBN / 2; i += 4)
          *reinterpret_cast<int4*>(dst + i) = make_int4(acc[i], acc[i + 1], acc[i + 2], acc[i + 3]);
      }
#pragma unroll
      for (int i = 0; i < kBN / 2; ++i) acc[i] = 0;
    }
    if (!ok && lane == 0) atomicExch(P.err, 1);
  }

  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols)
                 : "memory");
  }
  // paired: neither CTA leaves while the other may still send it a copy or a
  // stage release (every wait above is bounded, so both get here)
  if (P.pair) cluster_sync_all();
}

// ---------------------------------------------------------------------------
// Fold
// ---------------------------------------------------------------------------
struct OzakiFoldParams {
  int64_t m, n, k;
  int G, npass, b;
  int64_t m_pad, n_pad;
  const int32_t* C;      // [npass][G+1][m_pad][n_pad]
  const uint16_t* Y;     // CRT: [npass][nmod][m_pad][n_pad] reduced residue products (fp16 values)
  const int* S;          // row scales of op(A)
  const int* F;          // column scales of op(B)
  const uint32_t* fa;    // row special flags
  const uint32_t* fb;    // column special flags
  const q128* A;
  int64_t sai, sal;
  const q128* B;
  int64_t sbl, sbj;
  q128* Cout;
  int64_t sci, scj;
  q128 alpha, beta;
  const int* err;
  int* report;  // set to 1 when err is (mapped host memory; may be null)
  int T;        // CRT: operand truncation (the rounding is at 2^(S_i + F_j - 2T))
  // grouped problems: output row i is row i % 128 of list tile i / 128
  // (its problem, first local row and column, A and B tiles); the fields
  // A .. beta above are then unused
  const OzakiGroupTile* gtiles;
  const OzakiGroupProb* gprobs;
};

// Each thread folds four neighbouring columns j0..j0+3 of one row: one
// 16-byte load per diagonal plane (and k pass) feeds four Horner states, so
// a warp reads 512 contiguous bytes per plane; then one rounding and the
// reference epilogue per output.  (n_pad is a multiple of 256, so the four
// columns are always inside the planes; columns >= n are not written.)
template <int B>
__global__ void __launch_bounds__(256, 3) ozaki_fold_kernel(OzakiFoldParams P) {
  const int64_t j0 = ((int64_t)blockIdx.x * 32 + threadIdx.x) * 4;
  const int64_t i = (int64_t)blockIdx.y * 8 + threadIdx.y;
  if (i >= P.m || j0 >= P.n) return;
  const size_t plane4 = (size_t)P.m_pad * P.n_pad / 4;
  const size_t pass4 = (size_t)(P.G + 1) * plane4;
  const int4* src = reinterpret_cast<const int4*>(P.C + (size_t)i * P.n_pad + j0);
  fold192 f[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) fold_init(f[c]);
#pragma unroll 4
  for (int g = 0; g <= P.G; ++g) {
    const int4 v = __ldcs(src + g * plane4);
    int64_t t0 = v.x, t1 = v.y, t2 = v.z, t3 = v.w;
    for (int p = 1; p < P.npass; ++p) {
      const int4 w = __ldcs(src + p * pass4 + g * plane4);
      t0 += w.x;
      t1 += w.y;
      t2 += w.z;
      t3 += w.w;
    }
    fold_step_t<B>(f[0], t0);
    fold_step_t<B>(f[1], t1);
    fold_step_t<B>(f[2], t2);
    fold_step_t<B>(f[3], t3);
  }
  const bool failed = (P.err[0] | P.err[1] | P.err[2]) != 0;
  if (failed && P.report && i == 0 && j0 == 0) *reinterpret_cast<volatile int*>(P.report) = 1;
  const int Si = P.S[i];
  const uint32_t fai = P.fa[i];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const int64_t j = j0 + c;
    if (j < P.n && !(fai | P.fb[j])) {  // NaN / inf rows and columns: ozaki_special_kernel
      q128* cp = P.Cout + i * P.sci + j * P.scj;
      const q128 cold = *cp;
      const q128 sum = failed ? q_nan() : fold_round(f[c], ozaki_fold_exp(Si, P.F[j], P.G, B));
      *cp = q_epilogue(P.alpha, sum, P.beta, cold);
    }
  }
}

// Sums the residue planes of the k passes into the first pass's planes,
// modulo p_q (y is linear in C), for `rows` rows from Y (each plane `plane`
// values apart, a pass nmod planes), so that the reconstruction reads one
// pass.  The values are fp16 (integers below 2^11).
__global__ void __launch_bounds__(256)
    ozaki_crt_pass_sum_kernel(uint16_t* __restrict__ Y, int64_t rows, int64_t n_pad, int64_t plane, int nmod,
                              int npass, const __grid_constant__ CrtTable tab) {
  const int64_t per = rows * n_pad, total = (int64_t)nmod * per, pass = (int64_t)nmod * plane;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (int64_t)gridDim.x * blockDim.x) {
    const int q = (int)(x / per);
    uint16_t* y = Y + q * plane + (x - q * per);
    // fp16 values of integers below 2^11 (exact both ways)
    uint32_t v = (uint32_t)__half2float(__ushort_as_half(*y));
    for (int ps = 1; ps < npass; ++ps) v += (uint32_t)__half2float(__ushort_as_half(y[ps * pass]));
    *y = __half_as_ushort(__float2half_rn((float)crt_mod(v, tab.mod[q].p, tab.mod[q].magic)));
  }
}

// CRT reconstruction on the tensor cores (ozcrt.cuh, "Reconstruction on the
// tensor cores").  The product kernel stored y_q = (C_q mod p_q) u_q mod p_q
// as fp16 values (one k pass, or the passes summed by
// ozaki_crt_pass_sum_kernel).  Persistent CTAs of 4 warps walk tiles of
// 4 rows x 32 columns of C: warp w takes row 4t + w, lane l column l (one
// accumulator lane per output, M index 32w + l).  A tile's y values are
// copied (16-byte cp.async by every thread, 8 columns of one row of one
// plane each) straight into the MMA's A operand, per 16 moduli a block of
// [row][column group][modulus][8 columns] — an M-major operand without
// swizzle (8 outputs x 8 moduli per core matrix, the next 8 outputs 256
// bytes on, the next 8 moduli 128 bytes on); moduli beyond nmod are written
// as zeros.  Three buffers, fetched up to three tiles ahead; each thread
// fences its copies to the async proxy before the barrier after which the
// tile's MMAs are issued.  One thread issues one MMA per 16 moduli (M = 128, K = 16,
// N = crt_fold_n(NW)) of a tile against the byte table of M / p_q (K-major)
// into the CTA's accumulator.  Every thread reads its column sums (exact
// integers below 2^23, made integers by adding 2^23) into word sums
// (crt_fold_column); once all have, the next tile's MMAs are issued into the
// same accumulator and, while they run, each thread rounds X = Y - Q M once
// at 2^(S_i + F_j - 2T) and applies the reference epilogue.  One 64-column
// accumulator per CTA, five CTAs per SM (registers allow no more).  Every
// wait is bounded (1 s); on a timeout the CTA stops, waits for its copies
// and (bounded) for its MMAs in flight, records it in err[0] and frees its
// tensor memory (its remaining outputs stay unwritten, and the call reports
// the timeout).
constexpr int kFoldThreads = 128;
constexpr int kFoldTmemCols = 64;  // one accumulator (N <= 64 columns)
constexpr int kFoldCtasPerSm = 5;
constexpr int kFoldBufs = 3;
constexpr int kFoldBoxBytes = 8 * 16 * 4 * 4 * 2;                  // 16 moduli of a tile (4 KiB)
constexpr int kFoldBufBytes = kFoldBoxBytes * (kCrtMaxMods / 16);  // 12 KiB: every modulus of a tile
// M-major operand without swizzle: the descriptor's leading byte offset is
// the step between core matrices along K, its stride byte offset the step
// along M (the two swap roles against the K-major layout)
constexpr uint32_t kFoldALbo = 128;  // next 8 moduli (K)
constexpr uint32_t kFoldASbo = 256;  // next 8 outputs (M)
constexpr size_t kFoldSmem = 128 + kFoldBufs * kFoldBufBytes + kCrtFoldK * kCrtFoldMaxN * 2 + 128;  // about 43 KiB

template <int NW, bool kGrouped>
__global__ void __launch_bounds__(kFoldThreads, kFoldCtasPerSm)
    ozaki_crt_fold_tc_kernel(const __grid_constant__ OzakiFoldParams P, const __grid_constant__ CrtFoldTable tab) {
  constexpr int N = crt_fold_n(NW);
  extern __shared__ __align__(128) uint8_t fold_smem[];
  uint8_t* sbase = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(fold_smem) + 127) & ~(uintptr_t)127);
  uint8_t* ybuf = sbase;                                  // [3] A operands
  uint8_t* tbase = ybuf + kFoldBufs * kFoldBufBytes;      // the B table
  uint64_t* bar = reinterpret_cast<uint64_t*>(tbase + kCrtFoldK * kCrtFoldMaxN * 2);  // MMA completion
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nmod = tab.nmod, nboxes = (nmod + 15) / 16;
  for (int i = threadIdx.x; i < N * kCrtFoldK / 8; i += kFoldThreads)
    reinterpret_cast<uint4*>(tbase)[i] = reinterpret_cast<const uint4*>(tab.b)[i];
  fence_proxy_async_smem();
  if (threadIdx.x == 0) {
    mbar_init(smem_u32(bar), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kFoldTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  pdl_wait();
  pdl_trigger();
  const uint32_t tlane = tmem + ((uint32_t)(warp * 32) << 16);
  // kind::f16, fp32 D, fp16 A (M-major: bit 15) and B (K-major), N, M = 128
  constexpr uint32_t idesc = (1u << 4) | (1u << 15) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
  const uint32_t sb = smem_u32(tbase), lbo = (uint32_t)N * 16u, sy = smem_u32(ybuf);
  const bool failed = (P.err[0] | P.err[1] | P.err[2]) != 0;
  if (failed && P.report && blockIdx.x == 0 && threadIdx.x == 0) *reinterpret_cast<volatile int*>(P.report) = 1;

  // tiles t = blockIdx.x, + gridDim.x, ...: (row tile, column tile), by counting
  const int tiles_c = (int)((P.n + 31) / 32), tiles_r = (int)((P.m + 3) / 4);
  const int step_r = (int)gridDim.x / tiles_c, step_c = (int)gridDim.x % tiles_c;
  auto advance = [&](int& r_t, int& c_t) {
    c_t += step_c;
    r_t += step_r;
    if (c_t >= tiles_c) {
      c_t -= tiles_c;
      ++r_t;
    }
  };
  int tr = (int)blockIdx.x / tiles_c, tc = (int)blockIdx.x % tiles_c;  // the tile whose sums are read next
  int pr = tr, pc = tc;                                                 // the next tile to fetch
  uint32_t issued = 0, used = 0;  // tiles fetched / multiplied (buffer = count % 3)
  // every thread: its 16-byte pieces of the next tile (a box per 16 moduli,
  // [row][column group][modulus][8 columns] as above, 256 pieces per box:
  // 4 consecutive lanes read a row's 64 contiguous bytes of one plane) into
  // the tile's buffer, moduli beyond nmod as zeros; one commit group per
  // call, empty past the last tile
  const int64_t plane = P.m_pad * P.n_pad;
  auto fetch = [&]() {
    if (pr < tiles_r) {
      const uint32_t dst = sy + (issued % kFoldBufs) * kFoldBufBytes;
      const int64_t i0 = (int64_t)pr * 4, j0 = (int64_t)pc * 32;
      for (int p = threadIdx.x; p < nboxes * 256; p += kFoldThreads) {
        const int g = p & 3, m = (p >> 2) & 15, r = (p >> 6) & 3, x = p >> 8;
        const int q = 16 * x + m;
        const uint32_t so = (uint32_t)(x * kFoldBoxBytes + r * 1024 + g * 256 + m * 16);
        const uint16_t* src = P.Y + (q < nmod ? q * plane + (i0 + r) * P.n_pad + j0 + 8 * g : 0);
        cp_async16_zfill(dst + so, src, q < nmod ? 16u : 0u);
      }
      ++issued;
      advance(pr, pc);
    }
    cp_async_commit();
  };
  bool outstanding = false;  // thread 0: an MMA group issued and not yet seen complete
  // thread 0: tile `used`'s pieces are in and visible to the tensor cores;
  // its MMAs (one per box: moduli beyond nmod within a box are zero) into
  // the accumulator
  auto multiply = [&]() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t a0 = sy + (used % kFoldBufs) * kFoldBufBytes;
    for (int kt = 0; kt < nboxes; ++kt)
      mma_f16kind(tmem, smem_desc_noswizzle(a0 + kt * kFoldBoxBytes, kFoldALbo, kFoldASbo),
                  smem_desc_noswizzle(sb + 2 * kt * lbo, lbo, 128), idesc, kt ? 1u : 0u);
    mma_commit(smem_u32(bar));
    outstanding = true;
    ++used;
  };
  bool ok = true;
  // the first three tiles' pieces (three groups); the first tile's MMAs once
  // its group is in (the copies are generic-proxy writes: each thread fences
  // them to the async proxy before the barrier)
  for (int f = 0; f < kFoldBufs; ++f) fetch();
  cp_async_wait<kFoldBufs - 1>();
  fence_proxy_async_smem();
  __syncthreads();
  if (threadIdx.x == 0 && tr < tiles_r) multiply();
  // a tile's outputs (one per thread): where it goes, its scales and flags,
  // old C value (and, grouped, its problem's alpha and beta), loaded a tile
  // ahead of its rounding and combined only there, so that the loads are in
  // flight for a whole tile
  struct OutInfo {
    q128* cp;
    q128 cold;
    q128 al, be;
    int S, F;
    uint32_t fa, fb;
    bool mine;
  };
  auto out_info = [&](int r_t, int c_t) {
    OutInfo o;
    const int64_t i = (int64_t)r_t * 4 + warp, j = (int64_t)c_t * 32 + lane;
    if constexpr (kGrouped) {
      // m = 128 x tiles and n = 256: every (i, j) is inside the tile list
      const OzakiGroupTile gt = P.gtiles[i >> 7];
      const OzakiGroupProb& pr_ = P.gprobs[gt.prob];
      const int64_t li = gt.row0 + (i & 127), lj = gt.col0 + j;
      const int64_t ai = (int64_t)gt.a_tile * 128 + (i & 127), bj = (int64_t)gt.b_tile * 256 + j;
      o.mine = li < pr_.m && lj < pr_.n;
      o.cp = pr_.C + (o.mine ? li * pr_.sci + lj * pr_.scj : 0);
      o.fa = P.fa[ai];
      o.fb = P.fb[bj];
      o.S = P.S[ai];
      o.F = P.F[bj];
      o.al = pr_.alpha;
      o.be = pr_.beta;
    } else {
      o.mine = i < P.m && j < P.n;
      const int64_t ii = o.mine ? i : 0, jj = o.mine ? j : 0;
      o.cp = P.Cout + ii * P.sci + jj * P.scj;
      o.fa = P.fa[ii];
      o.fb = P.fb[jj];
      o.S = P.S[ii];
      o.F = P.F[jj];
      o.al = P.alpha;
      o.be = P.beta;
    }
    o.cold = ld_stream(o.cp);
    return o;
  };
  uint32_t mma_phase = 0;
  OutInfo cur;
  if (tr < tiles_r) cur = out_info(tr, tc);
  while (tr < tiles_r) {
    int nr = tr, nc = tc;  // the next tile
    advance(nr, nc);
    OutInfo nxt;
    if (nr < tiles_r) nxt = out_info(nr, nc);  // in flight while this tile is finished
    // this tile's column sums (every thread waits for the MMAs itself), read
    // into registers and folded into word sums
    CrtFoldAcc<NW> acc;
    crt_fold_init(acc);
    if (mbar_wait(smem_u32(bar), mma_phase & 1u)) {
      ++mma_phase;
      if (threadIdx.x == 0) outstanding = false;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int h = 0; h < (N + 31) / 32; ++h) {
        uint32_t z[32];
        tmem_ld16_nowait(tlane + (uint32_t)(32 * h), z);
        if (32 * h + 16 < N) tmem_ld16_nowait(tlane + (uint32_t)(32 * h + 16), z + 16);
        tmem_ld_wait();
        // two columns at a time (N is a multiple of 16): z + 2^23 in packed fp32
#pragma unroll
        for (int c = 0; c < 32; c += 2) {
          const int w = 32 * h + c;
          if (w < N) {
            uint32_t b0, b1;
            f32x2_unpack(f32x2_add(f32x2_pack(z[c], z[c + 1]), 0x4B0000004B000000ull), b0, b1);
            crt_fold_column(acc, w, b0, true);
            crt_fold_column(acc, w + 1, b1, true);
          }
        }
      }
    } else {
      ok = false;
    }
    // the next tile's pieces (the group before the newest) are in
    cp_async_wait<1>();
    fence_proxy_async_smem();
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    // the accumulator is read and this tile's y buffer is free: the next
    // tile's MMAs run while this tile is rounded, and the tile three ahead is
    // fetched into the free buffer
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    if (threadIdx.x == 0 && nr < tiles_r) multiply();
    fetch();
    // NaN / inf rows and columns (a flag set) are ozaki_special_kernel's
    if (cur.mine && (cur.fa | cur.fb) == 0u) {
      const q128 sum = failed ? q_nan() : crt_fold_finish(acc, tab.negM, cur.S + cur.F - 2 * P.T, true);
      if constexpr (kGrouped)
        *cur.cp = q_epilogue(cur.al, sum, cur.be, cur.cold);
      else
        *cur.cp = q_epilogue(P.alpha, sum, P.beta, cur.cold);
    }
    cur = nxt;
    tr = nr;
    tc = nc;
  }
  // after a timeout, the copies and MMAs still in flight are waited for
  // (bounded), so that none is outstanding when the tensor memory is freed
  const bool any_fail = __syncthreads_or(!ok) != 0;
  if (threadIdx.x == 0) {
    if (any_fail) {
      atomicExch(const_cast<int*>(P.err), 1);
      if (P.report) *reinterpret_cast<volatile int*>(P.report) = 1;
    }
    if (outstanding) mbar_wait(smem_u32(bar), mma_phase & 1u);
  }
  cp_async_wait<0>();
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kFoldTmemCols)
                 : "memory");
}

// Outputs in a row of op(A) or a column of op(B) that holds a NaN or an
// infinity: a direct wide-accumulator dot, so IEEE special-value semantics
// are kept (every such sum contains a special product, so it is exact).
// any[0] | any[1] (set by the scale kernels of both operands) says whether
// there is one at all; without, the launch returns at once.  Grid-stride
// over the outputs; threads of other outputs skip them.
__global__ void __launch_bounds__(256) ozaki_special_kernel(OzakiFoldParams P, const int* __restrict__ any) {
  pdl_wait();
  pdl_trigger();
  if ((any[0] | any[1]) == 0) return;
  const int64_t total = P.m * P.n;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = x / P.n, j = x % P.n;
    if (!(P.fa[i] | P.fb[j])) continue;
    q128* cp = P.Cout + i * P.sci + j * P.scj;
    wacc acc;
    wacc_init(acc);
    for (int64_t l = 0; l < P.k; ++l)
      wacc_add_product(acc, qop_unpack(ld_cached(P.A + i * P.sai + l * P.sal)),
                       qop_unpack(ld_cached(P.B + l * P.sbl + j * P.sbj)));
    *cp = q_epilogue(P.alpha, wacc_round(acc), P.beta, *cp);
  }
}

// The same for grouped problems: output (i, j) of the tile list's planes
// (row i % 128 of tile i / 128, column j) belongs to the tile's problem.
__global__ void __launch_bounds__(256)
    ozaki_special_grouped_kernel(OzakiFoldParams P, const int* __restrict__ any) {
  if ((any[0] | any[1]) == 0) return;
  const int64_t total = P.m * P.n;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = x / P.n, j = x % P.n;
    const OzakiGroupTile gt = P.gtiles[i >> 7];
    const int64_t ai = (int64_t)gt.a_tile * 128 + (i & 127), bj = (int64_t)gt.b_tile * 256 + j;
    if (!(P.fa[ai] | P.fb[bj])) continue;
    const OzakiGroupProb& pr = P.gprobs[gt.prob];
    const int64_t li = gt.row0 + (i & 127), lj = gt.col0 + j;
    if (li >= pr.m || lj >= pr.n) continue;
    q128* cp = pr.C + li * pr.sci + lj * pr.scj;
    wacc acc;
    wacc_init(acc);
    for (int64_t l = 0; l < pr.k; ++l)
      wacc_add_product(acc, qop_unpack(ld_cached(pr.A + li * pr.sai + l * pr.sal)),
                       qop_unpack(ld_cached(pr.B + l * pr.sbl + lj * pr.sbj)));
    *cp = q_epilogue(pr.alpha, wacc_round(acc), pr.beta, *cp);
  }
}

// Grouped problems: stacked row r (of a_all for r < rows_a, else of b_all)
// receives rows[r].len elements, rows[r].stride apart; one warp per row.
// The rest of the row stays as it is (zero).
__global__ void __launch_bounds__(256)
    ozaki_gather_kernel(const OzakiGroupRow* __restrict__ rows, int64_t nrows, int64_t rows_a, int64_t k_pad,
                        q128* __restrict__ a_all, q128* __restrict__ b_all) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x / 32);
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32; r < nrows; r += nw) {
    const OzakiGroupRow d = rows[r];
    q128* dst = r < rows_a ? a_all + r * k_pad : b_all + (r - rows_a) * k_pad;
    for (int64_t l = lane; l < d.len; l += 32) dst[l] = ld_stream(d.p + l * d.stride);
  }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
// 2-D tensor map (bf16, or fp16 for 9-bit digits) over D[rows][cols] with a
// (64 x box_rows) box, 128B swizzle.
static bool make_map(CUtensorMap* map, const void* D, int64_t rows, int64_t cols, int box_rows, bool f16) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
  cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, f16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                  const_cast<void*>(D), dims, strides, box,
                  estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

static int64_t rup(int64_t v, int64_t a) { return (v + a - 1) / a * a; }
static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// k-blocks per pass: a diagonal holds at most s pairs, each pair adds one
// exact chunk sum of magnitude <= 2^24 per chunk, and the int32 diagonal sum
// must stay below 2^31.
static int chunk_kblocks(int b) { return ozaki_exact_chunk(b) / kBK; }
static int pass_kblocks(int s, int b) {
  int chunks = (int)(((1ll << 31) - 1) / ((int64_t)s << 24));  // exact chunks per pass
  if (chunks < 1) chunks = 1;
  return chunks * chunk_kblocks(b);
}

// The CRT scheme's table for this call, or false for the digit pairs:
// scheme 1 asks for digit pairs; otherwise residues whenever the table for
// T = bits * digits - 1 and this k fits (ozcrt.cuh).
static bool ozaki_crt_table(int scheme, int digits, int bits, int64_t k, CrtTable& tab) {
  if (scheme == 1) return false;
  return crt_build(bits * digits - 1, k, tab);
}

struct OzakiLayout {
  int64_t m_pad, n_pad, k_pad;
  int s, b, G, npass;
  int nmod;   // CRT moduli (0: digit pairs)
  int kbp;    // k-blocks per pass
  size_t off_S, off_F, off_fa, off_fb, off_err, off_DA, off_DB, off_C, total;
};

// Scratch layout: s digit planes per operand and G + 1 = s diagonal planes
// per k pass, or (CRT) nmod residue planes per operand and per k pass.
static OzakiLayout ozaki_layout(int64_t m, int64_t n, int64_t k, int s, int b, int nmod) {
  OzakiLayout L;
  L.s = s;
  L.b = b;
  L.nmod = nmod;
  const int planes = nmod ? nmod : s;
  L.G = planes - 1;
  L.m_pad = rup(m, kBM);
  L.n_pad = rup(n, kBN);
  L.k_pad = rup(k, kBK);
  L.kbp = nmod ? kCrtPassK / kBK : pass_kblocks(s, b);
  const int64_t kbp = L.kbp;
  L.npass = (int)((L.k_pad / kBK + kbp - 1) / kbp);
  size_t o = 0;
  L.off_S = o;  o += align256((size_t)m * 4);
  L.off_F = o;  o += align256((size_t)n * 4);
  L.off_fa = o; o += align256((size_t)m * 4);
  L.off_fb = o; o += align256((size_t)n * 4);
  L.off_err = o; o += 256;
  L.off_DA = o; o += align256((size_t)planes * L.m_pad * L.k_pad * 2);
  L.off_DB = o; o += align256((size_t)planes * L.n_pad * L.k_pad * 2);
  L.off_C = o;  o += align256((size_t)L.npass * (L.G + 1) * L.m_pad * L.n_pad * (nmod ? 2 : 4));
  L.total = o;
  return L;
}

int ozaki_default_digits(int b) { return b == 7 ? 20 : (b == 8 ? 18 : 16); }
int ozaki_default_digit_bits() { return 9; }
int ozaki_digit_cap(int bits, int64_t k) { return ozaki_max_digits_for_k(bits, k); }

// ---- optional phase timing (CUDA events on the launching stream) ----------
namespace {
struct PhaseEvents {
  cudaEvent_t ev[4];  // start, after split, after digit products, after fold
  int64_t mma_flop_units;  // 2*m*n*k*pairs / 2^20, for the tensor roofline
  bool full;               // all four recorded (else only the products' two)
};
std::mutex g_prof_mu;
int g_prof_mode = 0;  // 0 off, 1 every phase, 2 the tensor-core products only
std::vector<PhaseEvents> g_prof_pending;
double g_prof_sum[3] = {0, 0, 0};
double g_prof_flop = 0;
int g_prof_calls = 0;

void prof_record(PhaseEvents* pe, int i, cudaStream_t st) {
  if (pe && (pe->full || i == 1 || i == 2)) cudaEventRecord(pe->ev[i], st);
}
}  // namespace

void ozaki_profile_enable(int mode) {
  std::lock_guard<std::mutex> l(g_prof_mu);
  g_prof_mode = mode;
}

// Sums of the phase times (ms) of the calls recorded since the last read:
// out[0] scale + split, out[1] digit products (tensor cores), out[2] fold;
// out[3] the algorithmic tensor flops of those calls (2*m*n*k*pairs).
int ozaki_profile_read(double* out, int* calls) {
  std::lock_guard<std::mutex> l(g_prof_mu);
  for (PhaseEvents& pe : g_prof_pending) {
    cudaEventSynchronize(pe.ev[pe.full ? 3 : 2]);
    float a = 0, b = 0, c = 0;
    if (pe.full) cudaEventElapsedTime(&a, pe.ev[0], pe.ev[1]);
    cudaEventElapsedTime(&b, pe.ev[1], pe.ev[2]);
    if (pe.full) cudaEventElapsedTime(&c, pe.ev[2], pe.ev[3]);
    g_prof_sum[0] += a;
    g_prof_sum[1] += b;
    g_prof_sum[2] += c;
    g_prof_flop += (double)pe.mma_flop_units * 1048576.0;
    ++g_prof_calls;
    for (int i = 0; i < 4; ++i) cudaEventDestroy(pe.ev[i]);
  }
  g_prof_pending.clear();
  out[0] = g_prof_sum[0];
  out[1] = g_prof_sum[1];
  out[2] = g_prof_sum[2];
  out[3] = g_prof_flop;
  *calls = g_prof_calls;
  g_prof_sum[0] = g_prof_sum[1] = g_prof_sum[2] = 0;
  g_prof_flop = 0;
  g_prof_calls = 0;
  return 0;
}

static int ozaki_nmod(int scheme, int digits, int bits, int64_t k) {
  CrtTable tab;
  return ozaki_crt_table(scheme, digits, bits, k, tab) ? tab.n : 0;
}

size_t ozaki_scratch_bytes(int64_t m, int64_t n, int64_t k, int digits, int bits, int scheme) {
  if (m <= 0 || n <= 0 || k <= 0) return 0;
  return ozaki_layout(m, n, k, digits, bits, ozaki_nmod(scheme, digits, bits, k)).total;
}

bool ozaki_uses_crt(int64_t k, int digits, int bits, int scheme) {
  return ozaki_nmod(scheme, digits, bits, k) > 0;
}

// Launches for the digit width b (7, 8 or 9).
static void launch_split(int b, dim3 grid, dim3 blk, cudaStream_t st, int64_t rows, int64_t cols,
                         int64_t rows_pad, int64_t cols_pad, int64_t plane, const q128* p, int64_t sr,
                         int64_t sc, const int* S, int s, uint16_t* D) {
  if (b == 7)
    ozaki_split_kernel<7><<<grid, blk, 0, st>>>(rows, cols, rows_pad, cols_pad, plane, p, sr, sc, S, s, D);
  else if (b == 8)
    ozaki_split_kernel<8><<<grid, blk, 0, st>>>(rows, cols, rows_pad, cols_pad, plane, p, sr, sc, S, s, D);
  else
    ozaki_split_kernel<9><<<grid, blk, 0, st>>>(rows, cols, rows_pad, cols_pad, plane, p, sr, sc, S, s, D);
}

static void launch_fold(int b, cudaStream_t st, const OzakiFoldParams& F) {
  dim3 blk(32, 8), grid((unsigned)((F.n + 127) / 128), (unsigned)((F.m + 7) / 8));
  if (b == 7)
    ozaki_fold_kernel<7><<<grid, blk, 0, st>>>(F);
  else if (b == 8)
    ozaki_fold_kernel<8><<<grid, blk, 0, st>>>(F);
  else
    ozaki_fold_kernel<9><<<grid, blk, 0, st>>>(F);
}

// CRT residues on the tensor cores: 18 bytes of V cover T <= 144, 24 cover
// T <= 191.  Persistent: four CTAs per SM (their tensor memory is 128
// columns each; the dynamic shared memory keeps a fifth off the SM).
// The side job of a split launch: row scales and flags of rows [0, rows) of
// a view with contiguous rows (row r at p + r * sr).
struct SplitSideScales {
  const q128* p;
  int64_t rows, cols, sr;
  int* S;
  uint32_t* flags;
  int* any;
};

static cudaError_t launch_crt_split(const CrtSplitTable& stab, cudaStream_t st, int64_t rows, int64_t cols,
                                    int64_t rows_pad, int64_t cols_pad, int64_t plane, const q128* p, int64_t sr,
                                    int64_t sc, const int* S, uint16_t* D, int* err,
                                    const SplitSideScales* side = nullptr, bool pdl = false) {
  CrtSplitParams P;
  P.rows = rows;
  P.cols = cols;
  P.rows_pad = rows_pad;
  P.cols_pad = cols_pad;
  P.plane = plane;
  P.p = p;
  P.sr = sr;
  P.sc = sc;
  P.S = S;
  P.err = err;
  P.D = D;
  const bool with_side = side && side->rows > 0;
  P.xs_p = with_side ? side->p : nullptr;
  P.xs_rows = with_side ? side->rows : 0;
  P.xs_cols = with_side ? side->cols : 0;
  P.xs_sr = with_side ? side->sr : 0;
  P.xs_S = with_side ? side->S : nullptr;
  P.xs_flags = with_side ? side->flags : nullptr;
  P.xs_any = with_side ? side->any : nullptr;
  const int64_t ntiles = (rows_pad / 4) * (cols_pad / 64);
  if (ntiles <= 0) return cudaSuccess;
  if (ntiles > INT32_MAX) return cudaErrorInvalidValue;
  const unsigned grid = (unsigned)std::min<int64_t>(ntiles, kSplitCtasPerSm * (int64_t)device_sm_count());
  const int threads = with_side ? kSplitSideThreads : kSplitThreads;
  if (stab.NB == 18)
    return launch_maybe_pdl(pdl, ozaki_crt_split_tc_kernel<18>, dim3(grid), dim3(threads), kSplitSmem, st, P, stab);
  return launch_maybe_pdl(pdl, ozaki_crt_split_tc_kernel<24>, dim3(grid), dim3(threads), kSplitSmem, st, P, stab);
}

// The reconstruction of rows [0, F.m) of F (its Y already offset to the
// band's first row; y_rows rows of each plane remain from there).
static cudaError_t launch_crt_fold(const CrtFoldTable& ft, cudaStream_t st, const OzakiFoldParams& F,
                                   int64_t y_rows, bool pdl = false) {
  const int64_t tiles = ((F.m + 3) / 4) * ((F.n + 31) / 32);
  if (tiles <= 0) return cudaSuccess;
  if (tiles > INT32_MAX || ft.N != crt_fold_n(ft.nw)) return cudaErrorInvalidValue;
  // the kernel reads each tile's y values as 16-byte pieces (8 columns of a
  // row of a plane): 16-byte aligned rows and planes, whole row tiles
  if (F.n_pad % 32 || y_rows % 4 || (reinterpret_cast<uintptr_t>(F.Y) & 15)) return cudaErrorInvalidValue;
  static std::atomic<bool> attr_set[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !attr_set[dev].load(std::memory_order_acquire)) {
    const void* k[6] = {(const void*)ozaki_crt_fold_tc_kernel<8, false>, (const void*)ozaki_crt_fold_tc_kernel<10, false>,
                        (const void*)ozaki_crt_fold_tc_kernel<12, false>, (const void*)ozaki_crt_fold_tc_kernel<8, true>,
                        (const void*)ozaki_crt_fold_tc_kernel<10, true>, (const void*)ozaki_crt_fold_tc_kernel<12, true>};
    for (int i = 0; i < 6; ++i) {
      cudaError_t e = cudaFuncSetAttribute(k[i], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFoldSmem);
      if (e != cudaSuccess) return e;
    }
    attr_set[dev].store(true, std::memory_order_release);
  }
  const unsigned grid = (unsigned)std::min<int64_t>(tiles, kFoldCtasPerSm * (int64_t)device_sm_count());
  const bool grouped = F.gtiles != nullptr;
  const dim3 g(grid), blk(kFoldThreads);
  if (ft.nw <= 8)
    return grouped ? launch_maybe_pdl(pdl, ozaki_crt_fold_tc_kernel<8, true>, g, blk, kFoldSmem, st, F, ft)
                   : launch_maybe_pdl(pdl, ozaki_crt_fold_tc_kernel<8, false>, g, blk, kFoldSmem, st, F, ft);
  if (ft.nw <= 10)
    return grouped ? launch_maybe_pdl(pdl, ozaki_crt_fold_tc_kernel<10, true>, g, blk, kFoldSmem, st, F, ft)
                   : launch_maybe_pdl(pdl, ozaki_crt_fold_tc_kernel<10, false>, g, blk, kFoldSmem, st, F, ft);
  return grouped ? launch_maybe_pdl(pdl, ozaki_crt_fold_tc_kernel<12, true>, g, blk, kFoldSmem, st, F, ft)
                 : launch_maybe_pdl(pdl, ozaki_crt_fold_tc_kernel<12, false>, g, blk, kFoldSmem, st, F, ft);
}

// Test hook of quadblas_debug_stall_next_call: set, the next Ozaki qgemm's
// products withhold one accumulator-full commit with 1 ms pipeline waits.
static std::atomic<int> g_stall_qgemm{0};
void ozaki_debug_stall_next() { g_stall_qgemm.store(1); }
static bool ozaki_take_stall() { return g_stall_qgemm.exchange(0) != 0; }

// Clusters of two product-kernel CTAs that can be resident at once on the
// current device (0 when clusters cannot be launched), looked up once.
static int mma_pair_clusters() {
  static std::atomic<int> cached[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
  int v = cached[dev].load(std::memory_order_relaxed);
  if (v) return v - 1;
  cudaError_t e = cudaFuncSetAttribute(ozaki_mma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMmaSmem);
  int n = 0;
  if (e == cudaSuccess) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(2);
    cfg.blockDim = dim3(kMmaThreads);
    cfg.dynamicSmemBytes = kMmaSmem;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 2;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    if (cudaOccupancyMaxActiveClusters(&n, (const void*)ozaki_mma_kernel, &cfg) != cudaSuccess) n = 0;
  }
  cudaGetLastError();
  cached[dev].store(n + 1, std::memory_order_relaxed);
  return n;
}

cudaError_t launch_gemm_ozaki(const GemmArgs& g, int digits, int bits, void* scratch, cudaStream_t st,
                              const OzakiOverlap* ov, int scheme, int* report) {
  if (g.m <= 0 || g.n <= 0 || g.k <= 0) return cudaSuccess;
  if ((bits < 7 || bits > 9) || digits < 2 || digits > ozaki_max_digits_for_k(bits, g.k))
    return cudaErrorInvalidValue;
  CrtTable tab;
  const bool crt = ozaki_crt_table(scheme, digits, bits, g.k, tab);
  CrtSplitTable stab;
  CrtFoldTable ftab;
  if (crt) {
    crt_split_table(tab, stab);
    crt_fold_table(tab, ftab);
  }
  OzakiLayout L = ozaki_layout(g.m, g.n, g.k, digits, bits, crt ? tab.n : 0);
  char* base = static_cast<char*>(scratch);
  int* S = reinterpret_cast<int*>(base + L.off_S);
  int* F = reinterpret_cast<int*>(base + L.off_F);
  uint32_t* fa = reinterpret_cast<uint32_t*>(base + L.off_fa);
  uint32_t* fb = reinterpret_cast<uint32_t*>(base + L.off_fb);
  int* err = reinterpret_cast<int*>(base + L.off_err);
  uint16_t* DA = reinterpret_cast<uint16_t*>(base + L.off_DA);
  uint16_t* DB = reinterpret_cast<uint16_t*>(base + L.off_DB);
  int32_t* Cg = reinterpret_cast<int32_t*>(base + L.off_C);
  uint16_t* Yq = reinterpret_cast<uint16_t*>(base + L.off_C);  // CRT: the same space as 16-bit planes
  cudaError_t e;
  const int sms = device_sm_count();
  PhaseEvents pev;
  PhaseEvents* pe = nullptr;
  {
    std::lock_guard<std::mutex> l(g_prof_mu);
    if (g_prof_mode) {
      bool okev = true;
      for (int i = 0; i < 4; ++i) okev = okev && cudaEventCreate(&pev.ev[i]) == cudaSuccess;
      if (okev) pe = &pev;
      pev.full = g_prof_mode == 1;
      int64_t pairs = crt ? (int64_t)tab.n : (int64_t)L.s * (L.s + 1) / 2;
      pev.mma_flop_units = (int64_t)((2.0 * g.m * g.n * g.k * pairs) / 1048576.0);
    }
  }
  prof_record(pe, 0, st);

  // 1. op(B) (its rows are the columns of op(B)): scales, flags and digits on
  // sb (the caller's stream for B when overlapping); the digit products wait
  // for it.
  cudaStream_t sb = ov ? ov->b_stream : st;
  const bool banded = ov && ov->a_rows;
  cudaStream_t sa = banded ? ov->a_stream : st;  // op(A): scales and digits, band by band
  // error words: [0] tensor-core products (main stream), [1] op(B)'s residue
  // split, [2] op(A)'s; [4], [5]: a NaN or infinity in op(B), in op(A).
  // On one stream one kernel sets the scales' starting values and resets
  // them; with a caller's streams each is reset on the stream of its writer.
  if (!ov) {
    // a programmatic dependent of whatever kernel came before in the stream:
    // it waits for it before its first write
    const int64_t mn = std::max<int64_t>(g.m, g.n);
    if ((e = launch_maybe_pdl(crt, ozaki_init_kernel, dim3((unsigned)((mn + 255) / 256)), dim3(256), 0, st, g.m, S,
                              fa, g.n, F, fb, err)) != cudaSuccess)
      return e;
  } else {
    ozaki_fill_kernel<<<(unsigned)((g.m + 255) / 256), 256, 0, sa>>>(g.m, S, fa);
    ozaki_fill_kernel<<<(unsigned)((g.n + 255) / 256), 256, 0, sb>>>(g.n, F, fb);
    if ((e = cudaMemsetAsync(err, 0, 4, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(err + 1, 0, 4, sb)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(err + 4, 0, 4, sb)) != cudaSuccess) return e;
  }
  const dim3 blk(32, 8);
  const int64_t plane_a = L.m_pad * L.k_pad, plane_b = L.n_pad * L.k_pad;
  // on one stream with op(A)'s rows contiguous, op(A)'s scales are taken by
  // a fifth warp of op(B)'s residue split instead of a launch of their own,
  // when that ends within the split: min(m, G) side warps (G CTAs in the
  // split's grid) each stream whole rows of op(A), 16 k bytes a row, at about
  // 3.4 GB/s, while the split moves about 80 n k bytes at about 5 TB/s, so
  // the side job fits when 300 m <= n min(m, G) (for m >= G: m <= about 2 n)
  const int64_t split_grid_b =
      std::min<int64_t>((L.n_pad / 4) * (L.k_pad / 64), (int64_t)kSplitCtasPerSm * sms);
  const bool a_side = crt && !ov && g.sal == 1 && 300 * g.m <= g.n * std::min<int64_t>(g.m, split_grid_b);
  // on one stream the residue scheme's kernels after the first are launched
  // as programmatic dependents (each waits for the one before it in its
  // pdl_wait; their launches overlap the tail of the kernel before)
  const bool pdl = crt && !ov;
  {
    if ((e = launch_scale(g.n, g.k, g.B, g.sbj, g.sbl, F, fb, err + 4, sms, sb, pdl)) != cudaSuccess) return e;
    dim3 gb((unsigned)(L.k_pad / 64), (unsigned)(L.n_pad / 8));
    const SplitSideScales side = {g.A, g.m, g.k, g.sai, S, fa, err + 5};
    if (crt)
      e = launch_crt_split(stab, sb, g.n, g.k, L.n_pad, L.k_pad, plane_b, g.B, g.sbj, g.sbl, F, DB, err + 1,
                           a_side ? &side : nullptr, pdl);
    else
      launch_split(L.b, gb, blk, sb, g.n, g.k, L.n_pad, L.k_pad, plane_b, g.B, g.sbj, g.sbl, F, L.s, DB);
    if (e != cudaSuccess || (e = cudaGetLastError()) != cudaSuccess) return e;
    if (ov) {
      if ((e = cudaEventRecord(ov->b_done, sb)) != cudaSuccess) return e;
      if ((e = cudaStreamWaitEvent(st, ov->b_done, 0)) != cudaSuccess) return e;
    }
  }
  // rows [r0, r1) of op(A) (r0, r1 multiples of the 128-row tile, r1 <= m_pad):
  // scales, flags and digits on sa; the main stream then waits for them
  auto cut_a = [&](int64_t r0, int64_t r1) -> cudaError_t {
    const int64_t rows = std::min(r1, g.m) - r0;
    cudaError_t ee;
    if (banded && ov->a_rows(ov->a_ctx, r0, r0 + rows, sa) != 0) return cudaErrorUnknown;
    if (ov && r0 == 0 &&
        ((ee = cudaMemsetAsync(err + 2, 0, 4, sa)) != cudaSuccess || (ee = cudaMemsetAsync(err + 5, 0, 4, sa)) != cudaSuccess))
      return ee;
    if (!a_side &&
        (ee = launch_scale(rows, g.k, g.A + r0 * g.sai, g.sai, g.sal, S + r0, fa + r0, err + 5, sms, sa, pdl)) !=
            cudaSuccess)
      return ee;
    dim3 ga((unsigned)(L.k_pad / 64), (unsigned)((r1 - r0) / 8));
    const q128* Ab = g.A + r0 * g.sai;
    ee = cudaSuccess;
    if (crt)
      ee = launch_crt_split(stab, sa, rows, g.k, r1 - r0, L.k_pad, plane_a, Ab, g.sai, g.sal, S + r0,
                            DA + r0 * L.k_pad, err + 2, nullptr, pdl);
    else
      launch_split(L.b, ga, blk, sa, rows, g.k, r1 - r0, L.k_pad, plane_a, Ab, g.sai, g.sal, S + r0, L.s,
                   DA + r0 * L.k_pad);
    if (ee != cudaSuccess || (ee = cudaGetLastError()) != cudaSuccess) return ee;
    if (banded) {
      if ((ee = cudaEventRecord(ov->a_done, sa)) != cudaSuccess) return ee;
      if ((ee = cudaStreamWaitEvent(st, ov->a_done, 0)) != cudaSuccess) return ee;
    }
    return cudaSuccess;
  };
  // 2. digit products on the tensor cores: one launch per (tile band, k pass).
  // Without a caller delivering op(A) by rows there is one band; with one,
  // the bands are whole waves of tiles (one tile per SM), at most 8, and
  // each band's digit products start as soon as its rows of op(A) are cut.
  CUtensorMap tmA, tmB, tmBh;
  if (!make_map(&tmA, DA, (int64_t)(L.G + 1) * L.m_pad, L.k_pad, kBM, crt || L.b == 9) ||
      !make_map(&tmB, DB, (int64_t)(L.G + 1) * L.n_pad, L.k_pad, kBN, crt || L.b == 9) ||
      !make_map(&tmBh, DB, (int64_t)(L.G + 1) * L.n_pad, L.k_pad, kBN / 2, crt || L.b == 9))
    return cudaErrorInvalidValue;
  static std::atomic<bool> attr_set[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !attr_set[dev].load(std::memory_order_acquire)) {
    if ((e = cudaFuncSetAttribute(ozaki_mma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kMmaSmem)) != cudaSuccess)
      return e;
    attr_set[dev].store(true, std::memory_order_release);
  }
  const int tiles_m = (int)(L.m_pad / kBM), tiles_n = (int)(L.n_pad / kBN);
  const int tiles = tiles_m * tiles_n;
  const int kb_total = (int)(L.k_pad / kBK), kbp = L.kbp;
  // paired CTAs (clusters of two sharing B) whenever there are two tile rows,
  // as many clusters as can be resident at once (the kernel is persistent)
  const int clusters = mma_pair_clusters();
  const bool stall = ozaki_take_stall();  // test hook: this call's products time out
  const bool pair = tiles_m >= 2 && clusters >= 1 && !stall;
  {
    static const bool debug = getenv("QBLAS_DEBUG") != nullptr;
    if (debug)
      fprintf(stderr, "qblas: Ozaki products %dx%d tiles, %s (%d resident clusters of two)\n", tiles_m, tiles_n,
              pair ? "paired CTAs" : "single CTAs", clusters);
  }
  int band_tiles = tiles;
  if (banded) {
    const int waves = (tiles + sms - 1) / sms;
    band_tiles = ((waves + 7) / 8) * sms;
    if (pair)
      band_tiles = (band_tiles + 2 * tiles_n - 1) / (2 * tiles_n) * (2 * tiles_n);  // whole tile-row pairs
    else
      band_tiles = (band_tiles + tiles_n - 1) / tiles_n * tiles_n;  // whole tile rows
  }
  // 3. fold + epilogue of rows [i0, i1) (the diagonal planes keep their
  // m_pad x n_pad shape); with a caller copying C out band by band, each
  // band is handed over as soon as it is folded
  OzakiFoldParams F2;
  F2.m = g.m; F2.n = g.n; F2.k = g.k;
  F2.G = L.G; F2.npass = L.npass; F2.b = L.b;
  F2.m_pad = L.m_pad; F2.n_pad = L.n_pad;
  F2.C = Cg; F2.Y = Yq; F2.S = S; F2.F = F; F2.fa = fa; F2.fb = fb;
  F2.A = g.A; F2.sai = g.sai; F2.sal = g.sal;
  F2.B = g.B; F2.sbl = g.sbl; F2.sbj = g.sbj;
  F2.Cout = g.C; F2.sci = g.sci; F2.scj = g.scj;
  F2.alpha = g.alpha; F2.beta = g.beta;
  F2.err = err;
  F2.report = report;
  F2.T = crt ? tab.T : 0;
  F2.gtiles = nullptr;
  F2.gprobs = nullptr;
  if ((g.m + 7) / 8 > 65535) return cudaErrorInvalidConfiguration;
  const bool fold_banded = ov && ov->band_done && g.scj == 1 && g.sci >= g.n && g.m >= 64;
  bool c_waited = false;
  auto fold_rows = [&](int64_t i0, int64_t i1) -> cudaError_t {
    cudaError_t ee;
    // C whole: one wait; C by bands: the latest record covers every row cut so far
    if (ov && (!c_waited || ov->c_banded)) {
      if ((ee = cudaStreamWaitEvent(st, ov->c_ready, 0)) != cudaSuccess) return ee;
      c_waited = true;
    }
    OzakiFoldParams Fb = F2;
    Fb.m = i1 - i0;
    Fb.C = Cg + (size_t)i0 * L.n_pad;
    Fb.Y = Yq + (size_t)i0 * L.n_pad;
    Fb.S = S + i0;
    Fb.fa = fa + i0;
    Fb.A = g.A + i0 * g.sai;
    Fb.Cout = g.C + i0 * g.sci;
    if (crt) {
      if (L.npass > 1) {  // the k passes' residues summed into the first
        const int64_t total = (int64_t)tab.n * Fb.m * L.n_pad;
        const unsigned gb = (unsigned)std::min<int64_t>((total + 255) / 256, (int64_t)sms * 8);
        ozaki_crt_pass_sum_kernel<<<gb, 256, 0, st>>>(Yq + (size_t)i0 * L.n_pad, Fb.m, L.n_pad,
                                                       L.m_pad * L.n_pad, tab.n, L.npass, tab);
        if ((ee = cudaGetLastError()) != cudaSuccess) return ee;
      }
      if ((ee = launch_crt_fold(ftab, st, Fb, L.m_pad - i0, pdl && L.npass == 1)) != cudaSuccess) return ee;
    } else {
      launch_fold(L.b, st, Fb);
    }
    if ((ee = cudaGetLastError()) != cudaSuccess) return ee;
    const unsigned sgrid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((Fb.m * g.n + 255) / 256, (int64_t)sms * 2));
    if ((ee = launch_maybe_pdl(pdl, ozaki_special_kernel, dim3(sgrid), dim3(256), 0, st, Fb,
                               (const int*)(err + 4))) != cudaSuccess)
      return ee;
    if ((ee = cudaGetLastError()) != cudaSuccess) return ee;
    if (fold_banded && ov->band_done(ov->band_ctx, i0, i1) != 0) return cudaErrorUnknown;
    return cudaSuccess;
  };

  int64_t rows_cut = 0, rows_folded = 0;
  for (int t0 = 0; t0 < tiles; t0 += band_tiles) {
    const int t1 = std::min(tiles, t0 + band_tiles);
    const int64_t rows_needed = std::min<int64_t>(L.m_pad, (int64_t)((t1 - 1) / tiles_n + 1) * kBM);
    if (rows_needed > rows_cut) {
      if ((e = cut_a(rows_cut, rows_needed)) != cudaSuccess) return e;
      rows_cut = rows_needed;
    }
    if (t0 == 0) prof_record(pe, 1, st);
    const int units = (L.G + 1) * (t1 - t0);
    for (int p = 0; p < L.npass; ++p) {
      OzakiMmaParams P;
      P.tiles_m = tiles_m;
      P.tiles_n = tiles_n;
      P.tile_begin = t0;
      P.tile_end = t1;
      P.idesc = (crt || L.b == 9) ? kIdescF16 : kIdescBf16;
      P.G = L.G;
      P.m_pad = (int)L.m_pad;
      P.n_pad = (int)L.n_pad;
      P.pa = (int)L.m_pad;
      P.pb = (int)L.n_pad;
      P.list = nullptr;
      P.kb_begin = p * kbp;
      P.kb_end = std::min(kb_total, (p + 1) * kbp);
      P.chunk_kb = crt ? chunk_kblocks(9) : chunk_kblocks(L.b);
      P.crt = crt ? 1 : 0;
      for (int q = 0; q < kCrtMaxMods; ++q) {
        const bool on = crt && q < tab.n;
        P.crt_p[q] = on ? tab.mod[q].p : 1u;
        P.crt_magic[q] = on ? tab.mod[q].magic : 0u;
        P.crt_K[q] = on ? tab.mod[q].K : 0u;
        P.crt_u[q] = on ? tab.mod[q].u : 0u;
      }
      P.C = Cg + (size_t)p * (L.G + 1) * L.m_pad * L.n_pad;
      P.Y = Yq + (size_t)p * (L.G + 1) * L.m_pad * L.n_pad;
      P.err = err;
      P.pair = pair ? 1 : 0;
      P.withhold = (stall && t0 == 0 && p == 0) ? 1 : 0;
      P.wait_ns = stall ? kStallWaitNs : kWaitLimitNs;
      if (pair) {
        const int vunits = (L.G + 1) * ((t1 - t0) / tiles_n + 1) / 2 * tiles_n;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)(2 * std::min(vunits, clusters)));
        cfg.blockDim = dim3(kMmaThreads);
        cfg.dynamicSmemBytes = kMmaSmem;
        cfg.stream = st;
        cudaLaunchAttribute at[2];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = 2;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[1].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = pdl ? 2 : 1;
        if ((e = cudaLaunchKernelEx(&cfg, ozaki_mma_kernel, tmA, tmB, tmBh, P)) != cudaSuccess) return e;
      } else {
        if ((e = launch_maybe_pdl(pdl, ozaki_mma_kernel, dim3((unsigned)std::min(units, sms)), dim3(kMmaThreads),
                                  kMmaSmem, st, tmA, tmB, tmBh, P)) != cudaSuccess)
          return e;
      }
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    // rows whose tiles are all done are folded before the next band
    // multiplies (so that their copy back overlaps the later bands), once
    // their rows of C are on the device: with C copied band by band
    // together with op(A)'s rows, at once; with C copied whole after op(A)'s
    // last rows, only then (a fold enqueued before that record would not
    // wait for C)
    if (banded && fold_banded && t1 < tiles && (ov->c_banded || rows_cut >= L.m_pad)) {
      const int64_t rows_done = std::min<int64_t>(g.m, (int64_t)(t1 / tiles_n) * kBM);
      if (rows_done > rows_folded) {
        if ((e = fold_rows(rows_folded, rows_done)) != cudaSuccess) return e;
        rows_folded = rows_done;
      }
    }
  }
  prof_record(pe, 2, st);
  // the remaining rows (all of them without banding), in up to 4 bands of at
  // least 1024 rows when the caller copies C out band by band (a few rows
  // left after the interleaved folds go in one band)
  {
    const int64_t left = g.m - rows_folded;
    const int64_t nb = fold_banded ? std::max<int64_t>(1, std::min<int64_t>(4, left / 1024)) : 1;
    const int64_t band_rows = ((left + nb - 1) / nb + 7) / 8 * 8;
    for (int64_t i0 = rows_folded; i0 < g.m; i0 += band_rows)
      if ((e = fold_rows(i0, std::min(g.m, i0 + band_rows))) != cudaSuccess) return e;
  }
  e = cudaSuccess;
  prof_record(pe, 3, st);
  if (pe) {
    std::lock_guard<std::mutex> l(g_prof_mu);
    g_prof_pending.push_back(pev);
  }
  return e;
}

size_t ozaki_error_flag_offset(int64_t m, int64_t n, int64_t k, int digits, int bits, int scheme) {
  return ozaki_layout(m, n, k, digits, bits, ozaki_nmod(scheme, digits, bits, k)).off_err;
}

// ---- grouped problems (residues) --------------------------------------------
// The single-call layout for the stacked operands (rows_a x k_pad and
// rows_b x k_pad), with the reduced products stored tile-major: nmod planes
// of (128 ntiles) x 256.  One k pass (k_pad <= 8192).
static bool ozaki_group_layout(int64_t rows_a, int64_t rows_b, int64_t k_pad, int64_t ntiles, int64_t k_max,
                               int digits, int bits, CrtTable& tab, OzakiLayout& L) {
  if (rows_a <= 0 || rows_b <= 0 || ntiles <= 0 || rows_a % kBM || rows_b % kBN || k_pad % kBK || k_pad <= 0 ||
      k_pad > kCrtPassK || k_max > k_pad || ntiles * kBM > INT32_MAX)
    return false;
  if (bits < 7 || bits > 9 || digits < 2 || digits > ozaki_max_digits_for_k(bits, k_max)) return false;
  if (!ozaki_crt_table(2, digits, bits, k_max, tab)) return false;
  L = ozaki_layout(rows_a, rows_b, k_pad, digits, bits, tab.n);
  L.total = L.off_C + align256((size_t)tab.n * (size_t)ntiles * kBM * kBN * 2);
  return true;
}

size_t ozaki_group_scratch_bytes(int64_t rows_a, int64_t rows_b, int64_t k_pad, int64_t ntiles, int64_t k_max,
                                 int digits, int bits) {
  CrtTable tab;
  OzakiLayout L;
  return ozaki_group_layout(rows_a, rows_b, k_pad, ntiles, k_max, digits, bits, tab, L) ? L.total : 0;
}

cudaError_t launch_gemm_ozaki_grouped(const OzakiGroup& Gp, cudaStream_t st) {
  CrtTable tab;
  OzakiLayout L;
  if (!ozaki_group_layout(Gp.rows_a, Gp.rows_b, Gp.k_pad, Gp.ntiles, Gp.k_max, Gp.digits, Gp.bits, tab, L))
    return cudaErrorInvalidValue;
  CrtSplitTable stab;
  CrtFoldTable ftab;
  crt_split_table(tab, stab);
  crt_fold_table(tab, ftab);
  char* base = static_cast<char*>(Gp.scratch);
  int* S = reinterpret_cast<int*>(base + L.off_S);
  int* F = reinterpret_cast<int*>(base + L.off_F);
  uint32_t* fa = reinterpret_cast<uint32_t*>(base + L.off_fa);
  uint32_t* fb = reinterpret_cast<uint32_t*>(base + L.off_fb);
  int* err = reinterpret_cast<int*>(base + L.off_err);
  uint16_t* DA = reinterpret_cast<uint16_t*>(base + L.off_DA);
  uint16_t* DB = reinterpret_cast<uint16_t*>(base + L.off_DB);
  uint16_t* Yq = reinterpret_cast<uint16_t*>(base + L.off_C);
  const int sms = device_sm_count();
  const int64_t ra = Gp.rows_a, rb = Gp.rows_b, kp = Gp.k_pad, nrows = ra + rb;
  cudaError_t e;
  // 1. the problems' rows into the stacked operands
  ozaki_gather_kernel<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((nrows + 7) / 8, (int64_t)sms * 8)), 256, 0,
                        st>>>(Gp.rows, nrows, ra, kp, Gp.a_all, Gp.b_all);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  // 2. scales, flags and residues of both (error words as in the single call)
  ozaki_fill_kernel<<<(unsigned)((ra + 255) / 256), 256, 0, st>>>(ra, S, fa);
  ozaki_fill_kernel<<<(unsigned)((rb + 255) / 256), 256, 0, st>>>(rb, F, fb);
  if ((e = cudaMemsetAsync(err, 0, 6 * sizeof(int), st)) != cudaSuccess) return e;
  launch_scale(rb, kp, Gp.b_all, kp, 1, F, fb, err + 4, sms, st);
  if ((e = launch_crt_split(stab, st, rb, kp, rb, kp, rb * kp, Gp.b_all, kp, 1, F, DB, err + 1)) != cudaSuccess)
    return e;
  launch_scale(ra, kp, Gp.a_all, kp, 1, S, fa, err + 5, sms, st);
  if ((e = launch_crt_split(stab, st, ra, kp, ra, kp, ra * kp, Gp.a_all, kp, 1, S, DA, err + 2)) != cudaSuccess)
    return e;
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  // 3. residue products over the tile list
  CUtensorMap tmA, tmB, tmBh;
  if (!make_map(&tmA, DA, (int64_t)tab.n * ra, kp, kBM, true) || !make_map(&tmB, DB, (int64_t)tab.n * rb, kp, kBN, true) ||
      !make_map(&tmBh, DB, (int64_t)tab.n * rb, kp, kBN / 2, true))
    return cudaErrorInvalidValue;
  if ((e = cudaFuncSetAttribute(ozaki_mma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMmaSmem)) !=
      cudaSuccess)
    return e;
  OzakiMmaParams P;
  P.tiles_m = (int)Gp.ntiles;
  P.tiles_n = 1;
  P.tile_begin = 0;
  P.tile_end = (int)Gp.ntiles;
  P.idesc = kIdescF16;
  P.G = tab.n - 1;
  P.m_pad = (int)(Gp.ntiles * kBM);
  P.n_pad = kBN;
  P.pa = (int)ra;
  P.pb = (int)rb;
  P.list = Gp.tiles;
  P.kb_begin = 0;
  P.kb_end = (int)(kp / kBK);
  P.chunk_kb = chunk_kblocks(9);
  P.crt = 1;
  for (int q = 0; q < kCrtMaxMods; ++q) {
    const bool on = q < tab.n;
    P.crt_p[q] = on ? tab.mod[q].p : 1u;
    P.crt_magic[q] = on ? tab.mod[q].magic : 0u;
    P.crt_K[q] = on ? tab.mod[q].K : 0u;
    P.crt_u[q] = on ? tab.mod[q].u : 0u;
  }
  P.C = nullptr;
  P.Y = Yq;
  P.err = err;
  P.pair = 0;
  P.withhold = 0;
  P.wait_ns = kWaitLimitNs;
  const int64_t units = (int64_t)tab.n * Gp.ntiles;
  ozaki_mma_kernel<<<(unsigned)std::min<int64_t>(units, sms), kMmaThreads, kMmaSmem, st>>>(tmA, tmB, tmBh, P);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  // 4. reconstruction and special values through the problems' C
  OzakiFoldParams F2 = {};
  F2.m = Gp.ntiles * kBM;
  F2.n = kBN;
  F2.k = Gp.k_max;
  F2.G = tab.n - 1;
  F2.npass = 1;
  F2.b = 9;
  F2.m_pad = Gp.ntiles * kBM;
  F2.n_pad = kBN;
  F2.Y = Yq;
  F2.S = S;
  F2.F = F;
  F2.fa = fa;
  F2.fb = fb;
  F2.Cout = nullptr;
  F2.err = err;
  F2.report = nullptr;
  F2.T = tab.T;
  F2.gtiles = Gp.tiles;
  F2.gprobs = Gp.probs;
  if ((e = launch_crt_fold(ftab, st, F2, F2.m_pad)) != cudaSuccess) return e;
  const unsigned sgrid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((F2.m * F2.n + 255) / 256, (int64_t)sms * 2));
  ozaki_special_grouped_kernel<<<sgrid, 256, 0, st>>>(F2, err + 4);
  return cudaGetLastError();
}

}  // namespace qb
