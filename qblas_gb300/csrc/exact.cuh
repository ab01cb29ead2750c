// Certified rounding of the wide accumulator, and an exact fallback.
//
// The wide accumulator (wacc.cuh) is exact until the sum falls below the
// 256-bit frame that the largest product anchors: every product, rescale
// and merge drops less than one unit of the frame's least significant bit,
// so for a sum of n products and g merges |S - W * 2^e| < (2n + 3g) units.
// wacc_round_certified() checks that no rounding boundary of binary128 lies
// within that distance of W * 2^e; then round(W * 2^e) is round(S), the
// correctly rounded exact sum.  Outputs that fail the check (sums that
// cancel far below their largest product, beyond what the frame holds) are
// recomputed exactly by a Kulisch accumulator: fixed-point digits spanning
// every product of two binary128 values, 32 bits per digit, kept in 64-bit
// carry-save form so that products can be added with plain integer adds
// (atomic adds in shared or global memory on the GPU).
//
// Compiled for the device and the host (the host versions are sequential).
#pragma once
#include "wacc.cuh"
#if defined(__CUDACC__)
#include "reduce.cuh"
#endif

namespace qb {

// ---------------------------------------------------------------------------
// Certificate
// ---------------------------------------------------------------------------
// out = round(W * 2^e) (as wacc_round); returns whether every value within
// err units of the frame's least significant bit rounds to the same out.
QB_HD bool wacc_round_certified(const wacc& a, uint64_t err, q128& out) {
  out = wacc_round(a);
  if (a.flags) return true;                 // NaN / infinity come from exact classes
  if (a.e == kWaccEmptyExp) return true;    // no finite nonzero product: exactly zero
  const uint32_t neg = a.w7 >> 31, mask = 0u - neg;
  u256 M = u256_make(((uint64_t)(a.w7 ^ mask) << 32) | (a.w6 ^ mask),
                     ((uint64_t)(a.w5 ^ mask) << 32) | (a.w4 ^ mask),
                     ((uint64_t)(a.w3 ^ mask) << 32) | (a.w2 ^ mask),
                     ((uint64_t)(a.w1 ^ mask) << 32) | (a.w0 ^ mask));
  if (neg) M = u256_add(M, u256_make(0, 0, 0, 1));
  if (u256_iszero(M)) return false;         // cancelled to within the truncation error
  const int L = 256 - clz256(M);            // bit length of |W|
  const int e_lead = a.e + L - 1;
  if (e_lead >= kExpField - kBias - 1) return false;  // at the overflow threshold
  int lsb = e_lead - 112;
  if (lsb < kLsbMin) lsb = kLsbMin;
  const int p = lsb - a.e;                  // the result's last bit is bit p of M
  if (p < 3 || p > 255) return false;
  if (p - 2 < 64 && (err >> (p - 2)) != 0) return false;  // need err < 2^(p-2)
  // rem = M mod 2^p, half = 2^(p-1); certified when |rem - half| > err
  bool st;
  u256 hi = u256_shr_sticky(M, p, st);
  u256 rem = u256_sub(M, u256_shl(hi, p), 0);
  u256 half = u256_shl(u256_make(0, 0, 0, 1), p - 1);
  u256 dist = u256_cmp(rem, half) >= 0 ? u256_sub(rem, half, 0) : u256_sub(half, rem, 0);
  return u256_cmp(dist, u256_make(0, 0, 0, err)) > 0;
}

// ---------------------------------------------------------------------------
// Kulisch accumulator
// ---------------------------------------------------------------------------
// Digit i holds bits [kKMinExp + 32 i, kKMinExp + 32 i + 32).  Products of
// two finite binary128 values lie in [2^-33242, 2^32768); their 256-bit
// significands (value = P * 2^(ea + eb), ea, eb >= -16621) start at digit 1
// or above and end below digit 2066.
constexpr int kKMinExp = -33280;
constexpr int kKDigits = 2080;

// Exact 256-bit product of the significands: limbs p[0..7].
QB_HD void mul128x128_full(const qop& a, const qop& b, uint32_t* p) {
  mul128x128_top224(a, b, p[1], p[2], p[3], p[4], p[5], p[6], p[7]);
  p[0] = a.m0 * b.m0;  // nothing carries out of limb 0
}

QB_HD void kulisch_digit_add(int64_t* d, int i, int64_t v) {
#if defined(__CUDA_ARCH__)
  atomicAdd(reinterpret_cast<unsigned long long*>(d + i), (unsigned long long)v);
#else
  d[i] += v;
#endif
}

// d += a * b for finite nonzero a, b; widens [lo, hi] to the digits touched.
QB_HD void kulisch_add_product(int64_t* d, const qop& a, const qop& b, int& lo, int& hi) {
  uint32_t p[8];
  mul128x128_full(a, b, p);
  const int pos = a.e + b.e - kKMinExp;
  const int idx = pos >> 5, sh = pos & 31;
  uint32_t q[9];
  if (sh == 0) {
    for (int t = 0; t < 8; ++t) q[t] = p[t];
    q[8] = 0;
  } else {
    q[0] = p[0] << sh;
    for (int t = 1; t < 8; ++t) q[t] = fshl32(p[t - 1], p[t], (uint32_t)sh);
    q[8] = p[7] >> (32 - sh);
  }
  const bool neg = (a.s ^ b.s) != 0;
  for (int t = 0; t < 9; ++t)
    if (q[t]) kulisch_digit_add(d, idx + t, neg ? -(int64_t)q[t] : (int64_t)q[t]);
  lo = idx < lo ? idx : lo;
  hi = idx + 8 > hi ? idx + 8 : hi;
}

// Carry-propagates digits [lo, hi] into [0, 2^32) and returns the final
// carry (0, or -1 when the total is negative: value = digits - 2^(32(hi+1))).
// Digits above hi must be zero; hi grows while the carry is neither 0 nor -1.
QB_HD int64_t kulisch_normalize(int64_t* d, int lo, int& hi) {
  int64_t carry = 0;
  for (int i = lo; i <= hi; ++i) {
    int64_t v = d[i] + carry;
    d[i] = v & 0xffffffffLL;
    carry = v >> 32;
  }
  while (carry != 0 && carry != -1 && hi + 1 < kKDigits) {
    ++hi;
    int64_t v = d[hi] + carry;
    d[hi] = v & 0xffffffffLL;
    carry = v >> 32;
  }
  return carry;
}

// Rounds the normalized digits [lo, hi] with final carry `carry` and the
// special-value flags (wacc encoding) to binary128.  Destroys the digits.
QB_HD q128 kulisch_round(int64_t* d, int lo, int hi, int64_t carry, uint32_t flags) {
  if ((flags & 1u) || ((flags & 6u) == 6u)) return q_nan();
  if (flags & 2u) return q_inf(0);
  if (flags & 4u) return q_inf(1);
  const uint32_t neg = carry < 0;
  if (neg) {  // magnitude = 2^(32(hi+1)) - digits
    uint64_t c = 1;
    for (int i = lo; i <= hi; ++i) {
      uint64_t v = (uint64_t)(uint32_t)~(uint32_t)d[i] + c;
      d[i] = (int64_t)(v & 0xffffffffull);
      c = v >> 32;
    }
  }
  int h = hi;
  while (h >= lo && d[h] == 0) --h;
  if (h < lo) return q_zero(0);
  uint64_t w[4] = {0, 0, 0, 0};
  for (int t = 0; t < 8; ++t) {
    int i = h - 7 + t;
    uint64_t v = (i >= lo) ? (uint64_t)d[i] : 0;
    w[t >> 1] |= v << (32 * (t & 1));
  }
  bool sticky = false;
  for (int i = lo; i < h - 7; ++i) sticky = sticky || d[i] != 0;
  return round_pack(neg, u256_make(w[3], w[2], w[1], w[0]), sticky, kKMinExp + 32 * (h - 7));
}

// ---------------------------------------------------------------------------
// Device side: a block-wide accumulator in shared memory, and the global
// state of a grid-wide exact dot
// ---------------------------------------------------------------------------
// Global state of a grid-wide exact sum: `need` is set by the kernel that
// found the fast result uncertified (which also resets the rest); every
// block adds its normalized digits with atomics, and the last block to
// arrive rounds.
struct ExactGlobal {
  int need;
  unsigned arrived;
  int lo, hi;
  uint32_t flags;
  int pad[3];
  int64_t d[kKDigits];
};

#if defined(__CUDACC__)
struct KulischBlock {
  int64_t d[kKDigits];
  int lo, hi;
  uint32_t flags;
};

// All threads of the block: empty accumulator.
__device__ __forceinline__ void kulisch_block_clear(KulischBlock& K) {
  for (int i = threadIdx.x; i < kKDigits; i += blockDim.x) K.d[i] = 0;
  if (threadIdx.x == 0) {
    K.lo = kKDigits;
    K.hi = -1;
    K.flags = 0;
  }
  __syncthreads();
}

// All threads of the block: K += sum of u(t) * v(t) over t = start, start +
// step, ... < n, where u(t) = U[t * su] and v(t) = W[t * sv]; ends with a
// barrier.
__device__ __forceinline__ void kulisch_block_add(KulischBlock& K, int64_t n, const q128* U, int64_t su,
                                                  const q128* W, int64_t sv, int64_t start,
                                                  int64_t step) {
  int lo = kKDigits, hi = -1;
  uint32_t fl = 0;
  for (int64_t t = start; t < n; t += step) {
    qop a = qop_unpack(ld_cached(U + t * su)), b = qop_unpack(ld_cached(W + t * sv));
    if ((a.cls | b.cls) != kClsFinite)
      fl |= special_product_flags(a, b);
    else
      kulisch_add_product(K.d, a, b, lo, hi);
  }
  if (hi >= lo) {
    atomicMin(&K.lo, lo);
    atomicMax(&K.hi, hi);
  }
  if (fl) atomicOr(&K.flags, fl);
  __syncthreads();
}

// Exact dot of one vector pair by the whole block (result valid in thread
// 0).  Ends with a barrier, so K can be reused.
__device__ __forceinline__ q128 block_exact_dot(KulischBlock& K, int64_t n, const q128* U, int64_t su,
                                                const q128* W, int64_t sv) {
  kulisch_block_clear(K);
  kulisch_block_add(K, n, U, su, W, sv, threadIdx.x, blockDim.x);
  q128 r = q_zero(0);
  if (threadIdx.x == 0) {
    int lo = K.lo, hi = K.hi;
    if (hi < lo) lo = hi = 0;
    int64_t c = kulisch_normalize(K.d, lo, hi);
    r = kulisch_round(K.d, lo, hi, c, K.flags);
  }
  __syncthreads();
  return r;
}

// Part of a grid-wide exact dot: this block's products (grid-stride over
// the n terms) are added into G; the last block to finish rounds the total
// and returns true in thread 0 with *out set.
__device__ __forceinline__ bool grid_exact_dot(KulischBlock& K, ExactGlobal* G, int64_t n, const q128* U,
                                               int64_t su, const q128* W, int64_t sv, q128* out) {
  kulisch_block_clear(K);
  kulisch_block_add(K, n, U, su, W, sv, (int64_t)blockIdx.x * blockDim.x + threadIdx.x,
                    (int64_t)gridDim.x * blockDim.x);
  bool last = false;
  if (threadIdx.x == 0) {
    int lo = K.lo, hi = K.hi;
    if (hi >= lo) {
      int64_t c = kulisch_normalize(K.d, lo, hi);
      for (int i = lo; i <= hi; ++i)
        if (K.d[i]) atomicAdd(reinterpret_cast<unsigned long long*>(G->d + i), (unsigned long long)K.d[i]);
      if (c && hi + 1 < kKDigits) {
        atomicAdd(reinterpret_cast<unsigned long long*>(G->d + hi + 1), (unsigned long long)c);
        ++hi;
      }
      atomicMin(&G->lo, lo);
      atomicMax(&G->hi, hi);
    }
    if (K.flags) atomicOr(&G->flags, K.flags);
    __threadfence();
    const unsigned prev = atomicAdd(&G->arrived, 1u);
    if (prev == gridDim.x - 1) {
      __threadfence();
      int glo = atomicAdd(&G->lo, 0), ghi = atomicAdd(&G->hi, 0);
      const uint32_t gfl = atomicOr(&G->flags, 0u);
      if (ghi < glo) glo = ghi = 0;
      for (int i = glo; i <= ghi; ++i) K.d[i] = __ldcg(G->d + i);
      int64_t c = kulisch_normalize(K.d, glo, ghi);
      *out = kulisch_round(K.d, glo, ghi, c, gfl);
      last = true;
    }
  }
  __syncthreads();
  return last;
}

// All threads of one block: prepares G for a grid-wide exact dot.
__device__ __forceinline__ void exact_global_reset(ExactGlobal* G) {
  for (int i = threadIdx.x; i < kKDigits; i += blockDim.x) G->d[i] = 0;
  if (threadIdx.x == 0) {
    G->arrived = 0;
    G->lo = kKDigits;
    G->hi = -1;
    G->flags = 0;
  }
}
#endif

}  // namespace qb
