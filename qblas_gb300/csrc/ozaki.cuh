// Ozaki-style error-free splitting of binary128 matrices into integer
// digits, and the fold of exact integer digit products back to binary128.
//
// A row i of op(A) is scaled by 2^S_i, S_i = max_l (exponent(a_il) + 1), so
// that |a_il| < 2^S_i, and written as the integer V = trunc(a_il *
// 2^(b*s - 1 - S_i)) (|V| < 2^(b*s - 1)), which is cut into s balanced
// base-2^b digits d_0 (most significant) .. d_{s-1}, |d_t| <= 2^(b-1):
//     a_il ~= 2^S_i * sum_t d_t * 2^(-(b-1) - b*t).
// Columns of op(B) are treated the same way (scale F_j).  With b = 8 the
// digits are integers in [-128, 128], exact in bf16, and a product of two
// is at most 2^14 in magnitude, so up to 1024 of them sum exactly in fp32
// (b = 7: [-64, 64], 2^12, 4096).
//
// For output (i, j), the digit products of diagonal g = t + u,
//     C_g(i, j) = sum_{t+u=g} sum_l dA_t(i, l) * dB_u(l, j),
// are exact integers, and
//     sum_l a_il b_lj ~= 2^(S_i + F_j - 2(b-1) - b*G) * sum_{g<=G} C_g 2^(b(G-g)),
// an exact 192-bit integer that is rounded once to binary128.  Pairs with
// t + u > G (G = s - 1) are dropped; the digit count s sets the accuracy.
#pragma once
#include <stdint.h>

#include "softquad.cuh"

namespace qb {

// Digit width b: 7 (|d| <= 64, fp32-exact over k-chunks of 4096) or 8
// (|d| <= 128, exact over k-chunks of 1024); both are exact in bf16.
constexpr int kOzakiMaxDigits = 22;  // V < 2^(b*s - 1) <= 2^175 (192-bit split)

// Largest digit count whose fold stays inside 192 bits:
// 31 (int32 diagonal) + b*(s-1) + 1 (sign) <= 191.
QB_HD int ozaki_max_digits(int b) { return b == 7 ? 22 : 20; }

// k-chunk (in elements) over which a digit product sums exactly in fp32:
// k * (2^(b-1))^2 <= 2^24.
QB_HD int ozaki_exact_chunk(int b) { return 1 << (24 - 2 * (b - 1)); }

// Exponent used for row/column scaling: exponent(x) + 1 for finite nonzero
// x (so |x| < 2^that), or a very small sentinel for zero.
constexpr int kOzakiScaleEmpty = -(1 << 29);

QB_HD int ozaki_exp_plus1(q128 a) {
  int be = q_bexp(a);
  if (be == kExpField) return kOzakiScaleEmpty;  // specials are flagged separately
  if (be != 0) return be - kBias + 1;
  uint64_t mh = a.hi & kMantHiMask, ml = a.lo;
  if ((mh | ml) == 0) return kOzakiScaleEmpty;
  int lz = mh ? clz64(mh) : 64 + clz64(ml);
  // leading one at bit (127 - lz) of (mh:ml); value = m * 2^(-16382-112)
  return (127 - lz) - 16382 - 112 + 1;
}

// Special-value flags of one element: bit0 NaN, bit1 +inf, bit2 -inf.
QB_HD uint32_t ozaki_special_flags(q128 a) {
  if (q_bexp(a) != kExpField) return 0u;
  if (q_isnan(a)) return 1u;
  return q_sign(a) ? 4u : 2u;
}

// The s balanced base-2^b digits of a for scale S, passed to emit(t, d_t)
// from the least significant (t = s-1) to the most significant (t = 0).
// Requires 1 <= s <= ozaki_max_digits(b); V is held in three 64-bit limbs
// (b*s - 1 <= 175 bits).
template <typename Emit>
QB_HD void ozaki_digits_emit(q128 a, int S, int s, int b, Emit emit) {
  int be = q_bexp(a);
  if (be == kExpField || q_iszero(a) || S == kOzakiScaleEmpty) {
    for (int t = s - 1; t >= 0; --t) emit(t, 0);
    return;
  }
  const bool neg = q_sign(a) != 0;
  uint64_t mh, ml;
  int E;
  q_unpack_norm(a, mh, ml, E);
  // V = trunc(m * 2^(E + b*s - 113 - S)); the shift is at most b*s - 114.
  int sh = E + b * s - 113 - S;
  uint64_t v0, v1, v2;
  if (sh >= 0) {
    u256 t = u256_shl(u256_make(0, 0, mh, ml), sh);
    v0 = t.w0;
    v1 = t.w1;
    v2 = t.w2;
  } else {
    bool st;
    u256 t = u256_shr_sticky(u256_make(0, 0, mh, ml), -sh, st);
    v0 = t.w0;
    v1 = t.w1;
    v2 = 0;
  }
  // balanced digits from the least significant end: d in [-2^(b-1), 2^(b-1) - 1],
  // top digit in [-2^(b-1), 2^(b-1)]
  const uint64_t mask = (1ull << b) - 1, half = 1ull << (b - 1);
  for (int t = s - 1; t >= 1; --t) {
    int d = (int)(v0 & mask);
    if ((uint64_t)d >= half) d -= (int)(1 << b);
    // V = (V - d) / 2^b (V stays non-negative)
    if (d >= 0) {
      uint64_t n0 = v0 - (uint64_t)d;
      uint64_t br = n0 > v0;
      v0 = n0;
      uint64_t n1 = v1 - br;
      br = br && v1 == 0;
      v1 = n1;
      v2 -= br;
    } else {
      uint64_t n0 = v0 + (uint64_t)(-d);
      uint64_t c = n0 < v0;
      v0 = n0;
      v1 += c;
      c = c && v1 == 0;
      v2 += c;
    }
    v0 = (v0 >> b) | (v1 << (64 - b));
    v1 = (v1 >> b) | (v2 << (64 - b));
    v2 >>= b;
    emit(t, neg ? -d : d);
  }
  // |V| < 2^(b*s-1) keeps the top digit in [0, 2^(b-1)]
  emit(0, neg ? -(int)v0 : (int)v0);
}

// The digits into an array: digits[t] for t < s.
QB_HD void ozaki_digits(q128 a, int S, int s, int b, int* digits) {
  ozaki_digits_emit(a, S, s, b, [&](int t, int d) { digits[t] = d; });
}

// 192-bit two's complement accumulator for the fold (Horner in base 2^b).
struct fold192 {
  uint64_t w0, w1, w2;
};

QB_HD void fold_init(fold192& f) { f.w0 = f.w1 = f.w2 = 0; }

// f = f * 2^b + v
QB_HD void fold_step(fold192& f, int64_t v, int b) {
  f.w2 = (f.w2 << b) | (f.w1 >> (64 - b));
  f.w1 = (f.w1 << b) | (f.w0 >> (64 - b));
  f.w0 = f.w0 << b;
  uint64_t vv = (uint64_t)v;
  uint64_t ext = v < 0 ? ~0ull : 0ull;
  uint64_t n0 = f.w0 + vv;
  uint64_t c0 = n0 < f.w0;
  f.w0 = n0;
  uint64_t t1 = f.w1 + ext;
  uint64_t c1 = t1 < f.w1;
  uint64_t n1 = t1 + c0;
  c1 += n1 < t1;
  f.w1 = n1;
  f.w2 = f.w2 + ext + c1;
}

// value = f * 2^e rounded to binary128
QB_HD q128 fold_round(const fold192& f, int e) {
  uint32_t neg = (uint32_t)(f.w2 >> 63);
  uint64_t a0 = f.w0, a1 = f.w1, a2 = f.w2;
  if (neg) {
    a0 = ~a0;
    a1 = ~a1;
    a2 = ~a2;
    a0 += 1;
    uint64_t c = a0 == 0;
    a1 += c;
    c = c && a1 == 0;
    a2 += c;
  }
  return round_pack(neg, u256_make(0, a2, a1, a0), false, e);
}

// Exponent of the fold's least significant bit for row scale S and column scale F.
QB_HD int ozaki_fold_exp(int S, int F, int G, int b) { return S + F - 2 * (b - 1) - b * G; }

}  // namespace qb
