// Level-3 soft-float kernel: qgemm, C = alpha * op(A) op(B) + beta * C.
//
// Replaces QuadBLAS::gemm / gemm_simple / the blocked macro and micro
// kernels (include/quadblas/algorithms/level3.hpp:17-336).  Each C(i,j) is
// the correctly rounded exact sum_l op(A)(i,l) op(B)(l,j) (wide accumulator,
// one rounding) followed by the reference epilogue
// C = fma(alpha, sum, beta * C) (level3.hpp:40,107,210).  The reference
// rounds once per k-panel of 126; this kernel rounds once in total, which is
// more accurate and within the k * u_q * sum|a b| reduction bound.
//
// Integer-pipe bound.  A CTA owns a 32 x 32 tile of C; its 256 threads each
// own a 2 x 2 block.  A and B k-slices of 16 are loaded once per CTA,
// unpacked (sign, exponent, significand shifted to bit 127) and staged in
// shared memory as structure-of-arrays, so the inner loop is the 128x128-bit
// product and the aligned add into the accumulator.
//
// Each rounding is certified (exact.cuh).  The few outputs whose sums
// cancel below what the 256-bit frame holds are listed in shared memory and
// recomputed exactly by the whole CTA after its tile (Kulisch accumulator in
// the shared memory that held the operand slices), so a call is one launch.
#include "exact.cuh"
#include "kernels.h"
#include "reduce.cuh"

namespace qb {

constexpr int kTM = 32, kTN = 32, kTK = 16;
constexpr int kGemmThreads = 256;

struct SoftTile {
  uint32_t m0[kTK][kTM], m1[kTK][kTM], m2[kTK][kTM], m3[kTK][kTM];
  int32_t e[kTK][kTM];
  uint32_t sc[kTK][kTM];  // sign | class << 1
};

__device__ __forceinline__ void tile_put(SoftTile& t, int kk, int idx, q128 v) {
  qop o = qop_unpack(v);
  t.m0[kk][idx] = o.m0;
  t.m1[kk][idx] = o.m1;
  t.m2[kk][idx] = o.m2;
  t.m3[kk][idx] = o.m3;
  t.e[kk][idx] = o.e;
  t.sc[kk][idx] = o.s | (o.cls << 1);
}

__device__ __forceinline__ qop tile_get(const SoftTile& t, int kk, int idx) {
  qop o;
  o.m0 = t.m0[kk][idx];
  o.m1 = t.m1[kk][idx];
  o.m2 = t.m2[kk][idx];
  o.m3 = t.m3[kk][idx];
  o.e = t.e[kk][idx];
  uint32_t sc = t.sc[kk][idx];
  o.s = sc & 1u;
  o.cls = sc >> 1;
  return o;
}

__global__ void __launch_bounds__(kGemmThreads)
    qgemm_soft_kernel(int64_t m, int64_t n, int64_t k, const q128* __restrict__ A, int64_t sai,
                      int64_t sal, const q128* __restrict__ B, int64_t sbl, int64_t sbj,
                      q128* __restrict__ C, int64_t sci, int64_t scj, q128 alpha, q128 beta) {
  // operand slices during the k-loop; the exact accumulator afterwards
  __shared__ union {
    struct {
      SoftTile a, b;
    } t;
    KulischBlock K;
  } sh;
  __shared__ int nlist;
  __shared__ short list[kTM * kTN];
  SoftTile& sA = sh.t.a;
  SoftTile& sB = sh.t.b;
  if (threadIdx.x == 0) nlist = 0;
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int64_t i0 = (int64_t)blockIdx.y * kTM, j0 = (int64_t)blockIdx.x * kTN;
  const q128 zero = q_zero(0);

  wacc c00, c01, c10, c11;
  wacc_init(c00);
  wacc_init(c01);
  wacc_init(c10);
  wacc_init(c11);

  for (int64_t l0 = 0; l0 < k; l0 += kTK) {
    // Stage op(A)[i0:i0+32, l0:l0+16]: element e -> (row e/16, kk e%16)
    // and op(B)[l0:l0+16, j0:j0+32]: element e -> (kk e/32, col e%32).
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      int e = tid + r * kGemmThreads;
      int ar = e >> 4, ak = e & 15;
      int64_t gi = i0 + ar, gl = l0 + ak;
      q128 av = (gi < m && gl < k) ? ld_cached(A + gi * sai + gl * sal) : zero;
      int bk = e >> 5, bc = e & 31;
      int64_t bl = l0 + bk, gj = j0 + bc;
      q128 bv = (bl < k && gj < n) ? ld_cached(B + bl * sbl + gj * sbj) : zero;
      tile_put(sA, ak, ar, av);
      tile_put(sB, bk, bc, bv);
    }
    __syncthreads();
#pragma unroll 2
    for (int kk = 0; kk < kTK; ++kk) {
      qop a0 = tile_get(sA, kk, 2 * ty), a1 = tile_get(sA, kk, 2 * ty + 1);
      qop b0 = tile_get(sB, kk, 2 * tx), b1 = tile_get(sB, kk, 2 * tx + 1);
      wacc_add_product(c00, a0, b0);
      wacc_add_product(c01, a0, b1);
      wacc_add_product(c10, a1, b0);
      wacc_add_product(c11, a1, b1);
    }
    __syncthreads();
  }

  const int64_t ia = i0 + 2 * ty, ja = j0 + 2 * tx;
  const uint64_t err = 2 * (uint64_t)k + 2;  // 2 units per product, no merges
  const wacc* cs[4] = {&c00, &c01, &c10, &c11};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int64_t i = ia + (q >> 1), j = ja + (q & 1);
    if (i < m && j < n) {
      q128 r;
      if (wacc_round_certified(*cs[q], err, r)) {
        q128* p = C + i * sci + j * scj;
        *p = q_epilogue(alpha, r, beta, *p);
      } else {
        list[atomicAdd(&nlist, 1)] = (short)((2 * ty + (q >> 1)) * kTN + 2 * tx + (q & 1));
      }
    }
  }
  __syncthreads();
  const int cnt = nlist;
  for (int t = 0; t < cnt; ++t) {
    const int64_t i = i0 + list[t] / kTN, j = j0 + list[t] % kTN;
    q128 r = block_exact_dot(sh.K, k, A + i * sai, sal, B + j * sbj, sbl);
    if (threadIdx.x == 0) {
      q128* p = C + i * sci + j * scj;
      *p = q_epilogue(alpha, r, beta, *p);
    }
  }
}

cudaError_t launch_gemm_softfloat(const GemmArgs& g, cudaStream_t s) {
  if (g.m <= 0 || g.n <= 0 || g.k <= 0) return cudaSuccess;
  int64_t gx = (g.n + kTN - 1) / kTN, gy = (g.m + kTM - 1) / kTM;
  if (gy > 65535) return cudaErrorInvalidConfiguration;
  dim3 grid((unsigned)gx, (unsigned)gy);
  qgemm_soft_kernel<<<grid, kGemmThreads, 0, s>>>(g.m, g.n, g.k, g.A, g.sai, g.sal, g.B, g.sbl, g.sbj,
                                                  g.C, g.sci, g.scj, g.alpha, g.beta);
  return cudaGetLastError();
}

}  // namespace qb
