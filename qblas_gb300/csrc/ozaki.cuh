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

// Digit width b: 7 (|d| <= 64, fp32-exact over k-chunks of 4096), 8
// (|d| <= 128, chunks of 1024), both exact in bf16; or 9 (|d| <= 256,
// chunks of 256), exact in fp16 (11-bit significand), whose 9-bit digits
// need fewer digit pairs for the same bits.
constexpr int kOzakiMaxDigits = 22;  // V < 2^(b*s - 1) <= 2^175 (192-bit split)

// Largest digit count whose fold stays inside 192 bits:
// 31 (int32 diagonal) + b*(s-1) + 1 (sign) <= 191.
template <int B>
struct OzakiMaxDigits {
  static constexpr int value = B == 7 ? 22 : (B == 8 ? 20 : 18);
};
QB_HD int ozaki_max_digits(int b) { return b == 7 ? 22 : (b == 8 ? 20 : 18); }

// Largest digit count for inner dimension k.  The fold value is
// sum_g C_g 2^(b(G-g)) with |C_g| <= (g+1) k 2^(2(b-1)), so
// |value| < 2 k 2^(2(b-1)) 2^(b(s-1)) (the geometric tail adds < 2^-6);
// it fits a 192-bit two's complement number when
// ceil(log2 k) + 2(b-1) + b(s-1) + 2 <= 191.
QB_HD int ozaki_max_digits_for_k(int b, int64_t k) {
  int lk = 0;
  while (lk < 63 && ((int64_t)1 << lk) < k) ++lk;
  int s = (191 - 2 - 2 * (b - 1) - lk) / b + 1;
  int cap = ozaki_max_digits(b);
  return s < cap ? s : cap;
}

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

// Bit field [p, p + B) of the 192-bit value (v2:v1:v0); p and B are
// compile-time constants after unrolling, so the shifts are constant.
template <int B>
QB_HD uint32_t ozaki_field(uint64_t v0, uint64_t v1, uint64_t v2, int p) {
  const uint64_t mask = (1ull << B) - 1;
  const int limb = p >> 6, off = p & 63;
  uint64_t lo = limb == 0 ? v0 : limb == 1 ? v1 : v2;
  uint64_t x = lo >> off;
  if (off + B > 64 && limb < 2) x |= (limb == 0 ? v1 : v2) << (64 - off);
  return (uint32_t)(x & mask);
}

// V = trunc(|a| * 2^(T - S)) (V < 2^T, T <= 191) as three 64-bit words and
// the sign of a; V = 0 for zero, NaN, infinity and an empty scale.
QB_HD void ozaki_scaled_bits(q128 a, int S, int T, uint64_t& v0, uint64_t& v1, uint64_t& v2, bool& neg) {
  v0 = v1 = v2 = 0;
  neg = q_sign(a) != 0;
  if (q_bexp(a) == kExpField || q_iszero(a) || S == kOzakiScaleEmpty) return;
  uint64_t mh, ml;
  int E;
  q_unpack_norm(a, mh, ml, E);
  // V = trunc(m * 2^(E + T - 112 - S)); the shift is at most T - 113.
  int sh = E + T - 112 - S;
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
  }
}

// The digit split's scaled integer: T = B*s - 1.
template <int B>
QB_HD void ozaki_scaled(q128 a, int S, int s, uint64_t& v0, uint64_t& v1, uint64_t& v2, bool& neg) {
  ozaki_scaled_bits(a, S, B * s - 1, v0, v1, v2, neg);
}

// Digit j (0 = least significant) of V from its raw field and the running
// carry; the top digit (j = s - 1) keeps r + carry.
template <int B>
QB_HD int ozaki_digit_step(uint64_t v0, uint64_t v1, uint64_t v2, int j, int s, int& carry) {
  int d = (int)ozaki_field<B>(v0, v1, v2, B * j) + carry;
  if (j < s - 1) {
    carry = d >= (1 << (B - 1));
    d -= carry << B;
  }
  return d;
}

// The s balanced base-2^B digits of a for scale S, passed to emit(t, d_t)
// from the least significant (t = s-1) to the most significant (t = 0).
// V = trunc(|a| * 2^(B*s - 1 - S)) < 2^(B*s - 1) is cut into its raw B-bit
// fields r_j (j = 0 least significant); a carry c (0 or 1) turns them into
// balanced digits: d_j = r_j + c - 2^B and c = 1 when r_j + c >= 2^(B-1),
// otherwise d_j = r_j + c and c = 0; the top digit takes r_{s-1} + c
// unchanged, which stays in [0, 2^(B-1)].  The signs follow a.
// Requires 1 <= s <= ozaki_max_digits(B).
template <int B, typename Emit>
QB_HD void ozaki_digits_emit(q128 a, int S, int s, Emit emit) {
  constexpr int kMax = OzakiMaxDigits<B>::value;
  uint64_t v0, v1, v2;
  bool neg;
  ozaki_scaled<B>(a, S, s, v0, v1, v2, neg);
  int carry = 0;
#pragma unroll
  for (int j = 0; j < kMax; ++j) {
    if (j < s) {
      int d = ozaki_digit_step<B>(v0, v1, v2, j, s, carry);
      emit(s - 1 - j, neg ? -d : d);
    }
  }
}

// The same for two values with one scale (two neighbours in a row):
// emit(t, d_t(a), d_t(b)).
template <int B, typename Emit2>
QB_HD void ozaki_digits_emit2(q128 a, q128 b, int S, int s, Emit2 emit) {
  constexpr int kMax = OzakiMaxDigits<B>::value;
  uint64_t a0, a1, a2, b0, b1, b2;
  bool na, nb;
  ozaki_scaled<B>(a, S, s, a0, a1, a2, na);
  ozaki_scaled<B>(b, S, s, b0, b1, b2, nb);
  int ca = 0, cb = 0;
#pragma unroll
  for (int j = 0; j < kMax; ++j) {
    if (j < s) {
      int da = ozaki_digit_step<B>(a0, a1, a2, j, s, ca);
      int db = ozaki_digit_step<B>(b0, b1, b2, j, s, cb);
      emit(s - 1 - j, na ? -da : da, nb ? -db : db);
    }
  }
}

// The digits into an array: digits[t] for t < s (b = 7, 8 or 9).
QB_HD void ozaki_digits(q128 a, int S, int s, int b, int* digits) {
  if (b == 7)
    ozaki_digits_emit<7>(a, S, s, [&](int t, int d) { digits[t] = d; });
  else if (b == 8)
    ozaki_digits_emit<8>(a, S, s, [&](int t, int d) { digits[t] = d; });
  else
    ozaki_digits_emit<9>(a, S, s, [&](int t, int d) { digits[t] = d; });
}

// 192-bit two's complement accumulator for the fold (Horner in base 2^b).
struct fold192 {
  uint64_t w0, w1, w2;
};

QB_HD void fold_init(fold192& f) { f.w0 = f.w1 = f.w2 = 0; }

// f = f * 2^B + v
template <int B>
QB_HD void fold_step_t(fold192& f, int64_t v) {
  const int b = B;
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

QB_HD void fold_step(fold192& f, int64_t v, int b) {
  if (b == 7)
    fold_step_t<7>(f, v);
  else if (b == 8)
    fold_step_t<8>(f, v);
  else
    fold_step_t<9>(f, v);
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
