// IEEE 754 binary128 ("quad") arithmetic on the integer pipes.
//
// Every function here is written from the IEEE 754-2019 definitions of
// addition, multiplication, fused multiply-add, square root and
// conversion, rounding to nearest with ties to even (RNE), with gradual
// underflow (subnormals), signed zeros, infinities and NaN.  It is
// compiled both as CUDA device code and as plain host C++, so that the
// same source can be checked bit-for-bit against a host binary128
// implementation on a machine without a GPU.
//
// The reference library delegates these operations to SLEEF's
// correctly rounded quad functions (Sleef_fmaq1_u05, Sleef_mulq1_u05,
// Sleef_addq1_u05, Sleef_sqrtq1_u05, Sleef_cast_from_doubleq1; called at
// include/quadblas/algorithms/level1.hpp:31,70,150,
// include/quadblas/algorithms/level2.hpp:43,48,65,71,79,
// include/quadblas/algorithms/level3.hpp:36,40,107 and
// include/quadblas/interface/c_interface.hpp:30,42,73,104).  SLEEF
// documents them as correctly rounded to within 0.5000000001 ulp, so an
// RNE-exact implementation returns the same bits for every finite result.
// NaN results are all returned as the canonical quiet NaN
// 0x7fff8000...0 (NaN payloads are not part of the contract).
//
// Layout of a binary128 value in memory (little-endian): word 0 holds the
// low 64 mantissa bits, word 1 holds sign (bit 63), the 15-bit biased
// exponent (bits 62..48) and the high 48 mantissa bits.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define QB_HD __host__ __device__ __forceinline__
#else
#define QB_HD static inline
#endif

namespace qb {

struct q128 {
  uint64_t lo, hi;
};

constexpr uint64_t kMantHiMask = 0x0000FFFFFFFFFFFFull;
constexpr uint64_t kHiddenBit = 0x0001000000000000ull;  // bit 112 of the significand
constexpr int kBias = 16383;
constexpr int kExpField = 0x7fff;
constexpr int kLsbMin = -16494;  // exponent of the least significant bit of the smallest subnormal

QB_HD q128 make_q(uint64_t hi, uint64_t lo) {
  q128 r;
  r.lo = lo;
  r.hi = hi;
  return r;
}
QB_HD q128 q_nan() { return make_q(0x7FFF800000000000ull, 0); }
QB_HD q128 q_inf(uint32_t s) { return make_q(((uint64_t)s << 63) | 0x7FFF000000000000ull, 0); }
QB_HD q128 q_zero(uint32_t s) { return make_q((uint64_t)s << 63, 0); }

QB_HD uint32_t q_sign(q128 a) { return (uint32_t)(a.hi >> 63); }
QB_HD int q_bexp(q128 a) { return (int)((a.hi >> 48) & 0x7fff); }
QB_HD bool q_isnan(q128 a) {
  return q_bexp(a) == kExpField && (((a.hi & kMantHiMask) | a.lo) != 0);
}
QB_HD bool q_isinf(q128 a) {
  return q_bexp(a) == kExpField && (((a.hi & kMantHiMask) | a.lo) == 0);
}
QB_HD bool q_iszero(q128 a) { return ((a.hi << 1) | a.lo) == 0; }

QB_HD void mul64(uint64_t a, uint64_t b, uint64_t& hi, uint64_t& lo) {
#if defined(__CUDA_ARCH__)
  lo = a * b;
  hi = __umul64hi(a, b);
#else
  unsigned __int128 p = (unsigned __int128)a * b;
  lo = (uint64_t)p;
  hi = (uint64_t)(p >> 64);
#endif
}

QB_HD int clz32(uint32_t x) {  // x != 0
#if defined(__CUDA_ARCH__)
  return __clz((int)x);
#else
  return __builtin_clz(x);
#endif
}

// ((hi:lo) << s) >> 32 for 0 <= s < 32
QB_HD uint32_t fshl32_any(uint32_t lo, uint32_t hi, int s) {
#if defined(__CUDA_ARCH__)
  return __funnelshift_l(lo, hi, (uint32_t)s);
#else
  return s ? (hi << s) | (lo >> (32 - s)) : hi;
#endif
}

QB_HD int clz64(uint64_t x) {  // x != 0
#if defined(__CUDA_ARCH__)
  return __clzll((long long)x);
#else
  return __builtin_clzll(x);
#endif
}

// 256-bit unsigned integer, w0 least significant.
struct u256 {
  uint64_t w0, w1, w2, w3;
};

QB_HD u256 u256_make(uint64_t w3, uint64_t w2, uint64_t w1, uint64_t w0) {
  u256 r;
  r.w0 = w0;
  r.w1 = w1;
  r.w2 = w2;
  r.w3 = w3;
  return r;
}
QB_HD bool u256_iszero(u256 x) { return (x.w0 | x.w1 | x.w2 | x.w3) == 0; }

QB_HD int clz256(u256 x) {  // x != 0
  if (x.w3) return clz64(x.w3);
  if (x.w2) return 64 + clz64(x.w2);
  if (x.w1) return 128 + clz64(x.w1);
  return 192 + clz64(x.w0);
}

// x >> s for s >= 0; st is set to whether any 1 bit was shifted out.
QB_HD u256 u256_shr_sticky(u256 x, int s, bool& st) {
  st = false;
  if (s <= 0) return x;
  if (s >= 256) {
    st = !u256_iszero(x);
    return u256_make(0, 0, 0, 0);
  }
  if (s >= 128) {
    st = st || ((x.w0 | x.w1) != 0);
    x.w0 = x.w2;
    x.w1 = x.w3;
    x.w2 = 0;
    x.w3 = 0;
    s -= 128;
  }
  if (s >= 64) {
    st = st || (x.w0 != 0);
    x.w0 = x.w1;
    x.w1 = x.w2;
    x.w2 = x.w3;
    x.w3 = 0;
    s -= 64;
  }
  if (s > 0) {
    st = st || ((x.w0 << (64 - s)) != 0);
    x.w0 = (x.w0 >> s) | (x.w1 << (64 - s));
    x.w1 = (x.w1 >> s) | (x.w2 << (64 - s));
    x.w2 = (x.w2 >> s) | (x.w3 << (64 - s));
    x.w3 >>= s;
  }
  return x;
}

// x << s for 0 <= s < 256 (bits shifted past bit 255 are discarded).
QB_HD u256 u256_shl(u256 x, int s) {
  if (s <= 0) return x;
  if (s >= 256) return u256_make(0, 0, 0, 0);
  if (s >= 128) {
    x.w3 = x.w1;
    x.w2 = x.w0;
    x.w1 = 0;
    x.w0 = 0;
    s -= 128;
  }
  if (s >= 64) {
    x.w3 = x.w2;
    x.w2 = x.w1;
    x.w1 = x.w0;
    x.w0 = 0;
    s -= 64;
  }
  if (s > 0) {
    x.w3 = (x.w3 << s) | (x.w2 >> (64 - s));
    x.w2 = (x.w2 << s) | (x.w1 >> (64 - s));
    x.w1 = (x.w1 << s) | (x.w0 >> (64 - s));
    x.w0 <<= s;
  }
  return x;
}

QB_HD u256 u256_add(u256 a, u256 b) {
  u256 r;
  r.w0 = a.w0 + b.w0;
  uint64_t c = r.w0 < a.w0;
  uint64_t t = a.w1 + c;
  uint64_t c1 = t < c;
  r.w1 = t + b.w1;
  c1 += r.w1 < t;
  t = a.w2 + c1;
  uint64_t c2 = t < c1;
  r.w2 = t + b.w2;
  c2 += r.w2 < t;
  r.w3 = a.w3 + b.w3 + c2;
  return r;
}

// a - b - borrow_in (borrow_in is 0 or 1); caller guarantees no underflow.
QB_HD u256 u256_sub(u256 a, u256 b, uint64_t borrow_in) {
  u256 r;
  uint64_t t = a.w0 - b.w0;
  uint64_t br = a.w0 < b.w0;
  r.w0 = t - borrow_in;
  br += t < borrow_in;
  t = a.w1 - b.w1;
  uint64_t br1 = a.w1 < b.w1;
  r.w1 = t - br;
  br1 += t < br;
  t = a.w2 - b.w2;
  uint64_t br2 = a.w2 < b.w2;
  r.w2 = t - br1;
  br2 += t < br1;
  r.w3 = a.w3 - b.w3 - br2;
  return r;
}

// -1, 0, 1 for a < b, a == b, a > b
QB_HD int u256_cmp(u256 a, u256 b) {
  if (a.w3 != b.w3) return a.w3 < b.w3 ? -1 : 1;
  if (a.w2 != b.w2) return a.w2 < b.w2 ? -1 : 1;
  if (a.w1 != b.w1) return a.w1 < b.w1 ? -1 : 1;
  if (a.w0 != b.w0) return a.w0 < b.w0 ? -1 : 1;
  return 0;
}

// Rounds (M + s*eps) * 2^f to binary128 with RNE, where M is a 256-bit
// magnitude, `sticky` says that a nonzero amount smaller than one unit of
// M's least significant bit was discarded below M, and s is the sign.
// Callers set sticky only when M's leading bit sits far above bit 113, so
// the round bit is always a real bit of M.
QB_HD q128 round_pack(uint32_t s, u256 M, bool sticky, int f) {
  if (u256_iszero(M)) return q_zero(s);
  int L = 255 - clz256(M);
  int e_lead = f + L;
  int lsb = e_lead - 112;
  if (lsb < kLsbMin) lsb = kLsbMin;
  int sh = lsb - f;
  uint64_t rh, rl;
  bool rbit, st;
  if (sh > 0) {
    u256 T = u256_shr_sticky(M, sh - 1, st);
    st = st || sticky;
    rbit = (T.w0 & 1) != 0;
    rl = (T.w0 >> 1) | (T.w1 << 63);
    rh = (T.w1 >> 1) | (T.w2 << 63);
  } else {
    u256 T = u256_shl(M, -sh);
    rbit = false;
    st = sticky;
    rl = T.w0;
    rh = T.w1;
  }
  if (rbit && (st || (rl & 1))) {
    rl += 1;
    if (rl == 0) rh += 1;
  }
  if (rh >> 49) {  // rounding carried into bit 113
    rl = (rl >> 1) | (rh << 63);
    rh >>= 1;
    lsb += 1;
  }
  if (rh & kHiddenBit) {
    int bexp = lsb + 112 + kBias;
    if (bexp >= kExpField) return q_inf(s);
    return make_q(((uint64_t)s << 63) | ((uint64_t)bexp << 48) | (rh & kMantHiMask), rl);
  }
  return make_q(((uint64_t)s << 63) | rh, rl);  // subnormal (or zero)
}

// Significand of a finite nonzero value normalised so that bit 112 is set:
// value = (mh:ml) * 2^(E - 112).
QB_HD void q_unpack_norm(q128 a, uint64_t& mh, uint64_t& ml, int& E) {
  int be = q_bexp(a);
  mh = a.hi & kMantHiMask;
  ml = a.lo;
  if (be != 0) {
    mh |= kHiddenBit;
    E = be - kBias;
    return;
  }
  int lz = mh ? clz64(mh) : 64 + clz64(ml);
  int sh = lz - 15;  // move the leading one from bit (127 - lz) to bit 112
  if (sh >= 64) {
    mh = ml << (sh - 64);
    ml = 0;
  } else if (sh > 0) {
    mh = (mh << sh) | (ml >> (64 - sh));
    ml <<= sh;
  }
  E = -16382 - sh;
}

// Exact 113 x 113 -> 226-bit product.
QB_HD u256 mul113(uint64_t ah, uint64_t al, uint64_t bh, uint64_t bl) {
  uint64_t h0, l0, h1, l1, h2, l2, h3, l3;
  mul64(al, bl, h0, l0);
  mul64(al, bh, h1, l1);
  mul64(ah, bl, h2, l2);
  mul64(ah, bh, h3, l3);
  u256 r;
  r.w0 = l0;
  uint64_t t = h0 + l1;
  uint64_t c = t < h0;
  r.w1 = t + l2;
  c += r.w1 < t;
  t = h1 + h2;
  uint64_t c2 = t < h1;
  t += l3;
  c2 += t < l3;
  r.w2 = t + c;
  c2 += r.w2 < t;
  r.w3 = h3 + c2;
  return r;
}

QB_HD q128 q_mul(q128 a, q128 b) {
  uint32_t s = q_sign(a) ^ q_sign(b);
  int ea = q_bexp(a), eb = q_bexp(b);
  bool za = q_iszero(a), zb = q_iszero(b);
  if (ea == kExpField || eb == kExpField) {
    if (q_isnan(a) || q_isnan(b)) return q_nan();
    if (za || zb) return q_nan();  // inf * 0
    return q_inf(s);
  }
  if (za || zb) return q_zero(s);
  uint64_t ah, al, bh, bl;
  int Ea, Eb;
  q_unpack_norm(a, ah, al, Ea);
  q_unpack_norm(b, bh, bl, Eb);
  return round_pack(s, mul113(ah, al, bh, bl), false, Ea + Eb - 224);
}

// Places x (a magnitude whose least significant bit has exponent `e`) into a
// frame whose bit 0 has exponent f: a left shift when e >= f, otherwise a
// right shift that records discarded bits in st.
QB_HD u256 place_in_frame(u256 x, int e, int f, bool& st) {
  int d = e - f;
  if (d >= 0) {
    st = false;
    return u256_shl(x, d);
  }
  return u256_shr_sticky(x, -d, st);
}

// Signed sum of two framed magnitudes.  At most one of st1/st2 is set, and
// only on the operand that is far smaller than the other.
QB_HD q128 framed_sum(uint32_t s1, u256 M1, bool st1, uint32_t s2, u256 M2, bool st2, int f) {
  if (s1 == s2) return round_pack(s1, u256_add(M1, M2), st1 || st2, f);
  if (st2) return round_pack(s1, u256_sub(M1, M2, 1), true, f);
  if (st1) return round_pack(s2, u256_sub(M2, M1, 1), true, f);
  int c = u256_cmp(M1, M2);
  if (c == 0) return q_zero(0);  // exact cancellation rounds to +0 under RNE
  if (c > 0) return round_pack(s1, u256_sub(M1, M2, 0), false, f);
  return round_pack(s2, u256_sub(M2, M1, 0), false, f);
}

QB_HD q128 q_add(q128 a, q128 b) {
  int ea = q_bexp(a), eb = q_bexp(b);
  uint32_t sa = q_sign(a), sb = q_sign(b);
  if (ea == kExpField || eb == kExpField) {
    if (q_isnan(a) || q_isnan(b)) return q_nan();
    if (ea == kExpField && eb == kExpField) return sa == sb ? a : q_nan();
    return ea == kExpField ? a : b;
  }
  bool za = q_iszero(a), zb = q_iszero(b);
  if (za && zb) return q_zero(sa & sb);
  if (za) return b;
  if (zb) return a;
  uint64_t ah, al, bh, bl;
  int Ea, Eb;
  q_unpack_norm(a, ah, al, Ea);
  q_unpack_norm(b, bh, bl, Eb);
  // Frame: the larger-exponent operand's leading bit at bit 253.
  int T = Ea > Eb ? Ea : Eb;
  int f = T - 253;
  bool st1, st2;
  u256 M1 = place_in_frame(u256_make(0, 0, ah, al), Ea - 112, f, st1);
  u256 M2 = place_in_frame(u256_make(0, 0, bh, bl), Eb - 112, f, st2);
  return framed_sum(sa, M1, st1, sb, M2, st2, f);
}

QB_HD q128 q_neg(q128 a) { return make_q(a.hi ^ 0x8000000000000000ull, a.lo); }
QB_HD q128 q_sub(q128 a, q128 b) {
  if (q_isnan(b)) return q_nan();
  return q_add(a, q_neg(b));
}

// a * b + c with a single rounding.
QB_HD q128 q_fma(q128 a, q128 b, q128 c) {
  uint32_t sa = q_sign(a), sb = q_sign(b), sc = q_sign(c);
  uint32_t sp = sa ^ sb;
  int ea = q_bexp(a), eb = q_bexp(b), ec = q_bexp(c);
  bool za = q_iszero(a), zb = q_iszero(b), zc = q_iszero(c);
  if (ea == kExpField || eb == kExpField || ec == kExpField) {
    if (q_isnan(a) || q_isnan(b) || q_isnan(c)) return q_nan();
    if (ea == kExpField || eb == kExpField) {
      if (za || zb) return q_nan();            // inf * 0
      if (ec == kExpField && sc != sp) return q_nan();  // inf - inf
      return q_inf(sp);
    }
    return c;  // finite product + inf
  }
  if (za || zb) {
    if (zc) return q_zero(sp & sc);
    return c;
  }
  uint64_t ah, al, bh, bl;
  int Ea, Eb;
  q_unpack_norm(a, ah, al, Ea);
  q_unpack_norm(b, bh, bl, Eb);
  u256 P = mul113(ah, al, bh, bl);
  int Ep = Ea + Eb - 224;  // exponent of P's least significant bit
  if (zc) return round_pack(sp, P, false, Ep);
  uint64_t ch, cl;
  int Ec;
  q_unpack_norm(c, ch, cl, Ec);
  int Lp = (P.w3 >> 33) ? 225 : 224;
  int Tp = Ep + Lp;
  int T = Tp > Ec ? Tp : Ec;
  int f = T - 253;
  bool st1, st2;
  u256 M1 = place_in_frame(P, Ep, f, st1);
  u256 M2 = place_in_frame(u256_make(0, 0, ch, cl), Ec - 112, f, st2);
  return framed_sum(sp, M1, st1, sc, M2, st2, f);
}

// Exact widening of an IEEE binary64 bit pattern.
QB_HD q128 q_from_double_bits(uint64_t d) {
  uint64_t s = d >> 63;
  int e = (int)((d >> 52) & 0x7ff);
  uint64_t m = d & 0x000FFFFFFFFFFFFFull;
  if (e == 0x7ff) {
    if (m) return q_nan();
    return q_inf((uint32_t)s);
  }
  if (e == 0) {
    if (m == 0) return q_zero((uint32_t)s);
    int lz = clz64(m);           // leading one at bit 63 - lz (<= 51)
    int sh = lz - 11;            // move it to bit 52
    m <<= sh;
    e = 1 - sh;
  }
  int bexp = e - 1023 + kBias;
  uint64_t frac = m & 0x000FFFFFFFFFFFFFull;  // 52 bits -> top of the 112-bit field
  return make_q((s << 63) | ((uint64_t)bexp << 48) | (frac >> 4), frac << 60);
}

// binary128 -> binary64 with RNE (host-side result conversion).
QB_HD uint64_t q_to_double_bits(q128 a) {
  uint64_t s = (uint64_t)q_sign(a) << 63;
  int be = q_bexp(a);
  if (be == kExpField) {
    if (q_isnan(a)) return 0x7FF8000000000000ull;
    return s | 0x7FF0000000000000ull;
  }
  if (q_iszero(a)) return s;
  uint64_t mh, ml;
  int E;
  q_unpack_norm(a, mh, ml, E);
  // value = m * 2^(E-112); target LSB exponent for binary64
  int lsb = E - 52;
  if (lsb < -1074) lsb = -1074;
  int sh = lsb - (E - 112);  // >= 60
  bool st;
  u256 T = u256_shr_sticky(u256_make(0, 0, mh, ml), sh - 1, st);
  bool rbit = T.w0 & 1;
  uint64_t r = (T.w0 >> 1) | (T.w1 << 63);
  if (rbit && (st || (r & 1))) r += 1;
  if (r >> 53) {
    r >>= 1;
    lsb += 1;
  }
  if (r >> 52) {
    int bexp = lsb + 52 + 1023;
    if (bexp >= 0x7ff) return s | 0x7FF0000000000000ull;
    return s | ((uint64_t)bexp << 52) | (r & 0x000FFFFFFFFFFFFFull);
  }
  return s | r;
}

// Integer square root helper: floor(sqrt(x)) of a 256-bit value by the
// digit-by-digit (restoring) method, two result bits per step position.
// Returns the root in (rh:rl) and sets `exact` if the remainder is zero.
QB_HD void isqrt256(u256 x, uint64_t& rh, uint64_t& rl, bool& exact) {
  // root fits in 128 bits
  u256 rem = u256_make(0, 0, 0, 0);
  uint64_t qh = 0, ql = 0;
  for (int i = 127; i >= 0; --i) {
    // bring down two bits of x: bits (2i+1, 2i)
    int b = 2 * i;
    uint64_t w = b >= 192 ? x.w3 : b >= 128 ? x.w2 : b >= 64 ? x.w1 : x.w0;
    uint64_t two = (w >> (b & 63)) & 3;
    rem = u256_shl(rem, 2);
    rem.w0 |= two;
    // trial = 4q + 1 where q is the current root (as 130-bit)
    u256 trial = u256_make(0, qh >> 62, (qh << 2) | (ql >> 62), (ql << 2) | 1);
    uint64_t nqh = (qh << 1) | (ql >> 63), nql = ql << 1;
    if (u256_cmp(rem, trial) >= 0) {
      rem = u256_sub(rem, trial, 0);
      nql |= 1;
    }
    qh = nqh;
    ql = nql;
  }
  rh = qh;
  rl = ql;
  exact = u256_iszero(rem);
}

QB_HD q128 q_sqrt(q128 a) {
  uint32_t s = q_sign(a);
  int be = q_bexp(a);
  if (q_isnan(a)) return q_nan();
  if (q_iszero(a)) return a;  // sqrt(+-0) = +-0
  if (s) return q_nan();
  if (be == kExpField) return a;  // +inf
  uint64_t mh, ml;
  int E;
  q_unpack_norm(a, mh, ml, E);
  // value = m * 2^(E-112), m in [2^112, 2^113).  Write value = X * 2^(2k)
  // with X = m << t (t = 116 or 117, chosen to make the remaining exponent
  // even), so that floor(sqrt(X)) has exactly 115 bits: the 113 result
  // bits, the round bit and one more, with the remainder as sticky.
  int e0 = E - 112;
  int t = 116;
  if ((e0 - t) & 1) t += 1;
  u256 X = u256_shl(u256_make(0, 0, mh, ml), t);
  int k2 = e0 - t;            // value = X * 2^k2, k2 even
  uint64_t rh, rl;
  bool exact;
  isqrt256(X, rh, rl, exact);
  // sqrt(value) = (r + frac) * 2^(k2/2); r has 113..114 bits, frac > 0 iff !exact
  u256 R = u256_make(0, 0, rh, rl);
  return round_pack(0, R, !exact, k2 / 2);
}

// The reference epilogue y = fma(alpha, sum, beta * y) (level2.hpp:48,
// level3.hpp:107).  fma(1, s, t) is s + t with one rounding, so alpha == 1
// takes the cheaper addition; the result bits are identical.
QB_HD q128 q_epilogue(q128 alpha, q128 sum, q128 beta, q128 y) {
  const bool one = alpha.hi == 0x3FFF000000000000ull && alpha.lo == 0;
  if (q_iszero(beta) && q_bexp(y) != kExpField) {
    // beta * y is a zero of sign sb ^ sy (y finite), so fma(alpha, sum, t)
    // is the rounded product alpha * sum, except where that product is
    // exactly zero: then IEEE addition of two zeros gives -0 only for two -0
    // (round to nearest).  NaN and infinite products are unchanged by a zero.
    const uint32_t st = q_sign(beta) ^ q_sign(y);
    if (one) {
      if (q_isnan(sum)) return q_nan();
      return q_iszero(sum) ? q_zero(q_sign(sum) & st) : sum;
    }
    const q128 p = q_mul(alpha, sum);
    if (q_bexp(p) == kExpField) return p;
    return (q_iszero(alpha) || q_iszero(sum)) ? q_zero(q_sign(p) & st) : p;
  }
  q128 t = q_mul(beta, y);
  if (one) return q_add(sum, t);
  return q_fma(alpha, sum, t);
}

}  // namespace qb
