// Ozaki-split qgemv: the arithmetic shared by the kernels (ozgemv.cu) and
// the host tests.
//
// y_i = sum_j A(i,j) x_j is cut into chunks of kOgChunk = 32 columns.  In a
// chunk, row i's elements are scaled by their largest lead-bit exponent E
// (subnormals and zeros counted as -16382) and x's by its largest F, and
// each element a becomes a 144-bit fixed-point integer
//   V = floor(|a| / 2^(E - 141)),   V < 2^142,
// cut into 18 balanced 8-bit digits d_0 (most significant) .. d_17:
//   V = sum_t d_t 256^(17 - t),   d_t in [-128, 128),
// and a's digits are sign(a) * d_t.  The d_t are the bytes of W = V + R,
// R = sum_t 128 * 256^t, minus 128: as fp16 values a digit is
// sign * ((1024 + byte) - 1152), one byte select and one fused multiply-add
// of a pair of halves, exact.
//
// Digit products are exact in fp16 x fp16 -> fp32 (|d_t d_u| <= 2^14), and a
// chunk's diagonal sums D_g = sum_j sum_{t+u=g} d_t(a_j) d_u(x_j) stay below
// 18 * 32 * 2^14 < 2^24, so tensor-core fp32 accumulation is exact.  Then
//   sum_j a'_j x'_j = 2^(E + F - 282) sum_g D_g 256^(34 - g)
// and the chunk contributes T * 2^(E + F - 162) with
//   T = sum_{g<20} D_g 256^(19 - g)   (|T| < 2^177: six 32-bit words).
// Its error against the exact sum_j a_j x_j is below 2^(E + F - 133):
// operand truncation |a x - a' x'| < 2^(E-141) 2^(F+1) + 2^(E+1) 2^(F-141)
// per product (32 * 2^(E+F-139) per chunk) plus the dropped diagonals
// g >= 20 (< 2^(E + F - 146.7)).
#pragma once
#include "wacc.cuh"

namespace qb {

constexpr int kOgChunk = 32;        // columns per exact fp32 accumulation
constexpr int kOgPlanes = 18;       // 8-bit digits per element
constexpr int kOgDiags = 20;        // diagonals folded into T
constexpr int kOgFoldShift = 162;   // chunk value = T * 2^(E + F - 162)
constexpr int kOgErrShift = 133;    // |chunk error| < 2^(E + F - 133)
constexpr int kOgNoExp = -(1 << 20);  // x chunk without a nonzero element

// Balanced ranges of (row tile, chunk) items over G CTAs: CTA b takes items
// [og_range_begin(b), og_range_begin(b + 1)); og_cta_of(X) is the CTA whose
// range holds item X (the smallest b with og_range_begin(b + 1) > X).
QB_HD int64_t og_range_begin(int64_t work, int64_t G, int64_t b) { return work * b / G; }
QB_HD int64_t og_cta_of(int64_t work, int64_t G, int64_t X) { return ((X + 1) * G + work - 1) / work - 1; }

// Lead-bit exponent of an element from its top 32 bits (sign, exponent,
// fraction bits 111..96); zeros and subnormals give -16382 (an upper bound).
QB_HD int og_lead_top(uint32_t top) {
  const uint32_t be = (top >> 16) & 0x7FFFu;
  return (int)(be ? be : 1u) - 16383;
}

QB_HD bool og_special_top(uint32_t top) { return ((top >> 16) & 0x7FFFu) == 0x7FFFu; }

// Shift that places an element's significand in the window of chunk
// exponent E: V = (M << 32) >> og_shift(E, w3), M the 113-bit significand.
// At least 3 (E is at least the element's lead exponent); from 160 on, V = 0.
QB_HD int og_shift(int E, uint32_t w3) {
  const uint32_t be = (w3 >> 16) & 0x7FFFu;
  return E + 16386 - (int)(be > 1u ? be : 1u);
}

// W = R + V for the element with 32-bit words w0 (least significant) .. w3
// and shift s = og_shift(E, w3) (hidden bit set iff the exponent field is
// nonzero).  W < 2^144: five words, W[4] < 2^16.  Branch-free (lanes of a
// warp hold elements of different exponents): the word part of the shift is
// three select levels; kShort drops the level for 4 words and the clamp, valid
// when s < 128.  NaN and infinity give bounded garbage (their rows are
// recomputed exactly).
template <bool kShort>
QB_HD void og_window_s(uint32_t w0, uint32_t w1, uint32_t w2, uint32_t w3, int s, uint32_t (&W)[5]) {
  const uint32_t be = (w3 >> 16) & 0x7FFFu;
  const uint32_t hb = be + 0xFFFFu;  // bit 16 set iff be != 0 (hb < 2^17)
  const uint32_t m3 = (w3 & 0xFFFFu) | (hb & 0x10000u);
  if (!kShort) s = s < 160 ? s : 160;
  const uint32_t b = (uint32_t)s & 31u, k = (uint32_t)s >> 5;
  uint32_t y0 = fshr32(0u, w0, b), y1 = fshr32(w0, w1, b), y2 = fshr32(w1, w2, b), y3 = fshr32(w2, m3, b),
           y4 = m3 >> b;
  const bool k2 = (k & 2u) != 0, k1 = (k & 1u) != 0;
  if (!kShort) {
    const bool k4 = (k & 4u) != 0;
    y0 = k4 ? y4 : y0;
    y1 = k4 ? 0u : y1;
    y2 = k4 ? 0u : y2;
    y3 = k4 ? 0u : y3;
    y4 = k4 ? 0u : y4;
  }
  y0 = k2 ? y2 : y0;
  y1 = k2 ? y3 : y1;
  y2 = k2 ? y4 : y2;
  y3 = k2 ? 0u : y3;
  y4 = k2 ? 0u : y4;
  y0 = k1 ? y1 : y0;
  y1 = k1 ? y2 : y1;
  y2 = k1 ? y3 : y2;
  y3 = k1 ? y4 : y3;
  y4 = k1 ? 0u : y4;
#if defined(__CUDA_ARCH__)
  uint32_t r0, r1, r2, r3, r4;
  asm("add.cc.u32  %0, %5, 0x80808080;\n\t"
      "addc.cc.u32 %1, %6, 0x80808080;\n\t"
      "addc.cc.u32 %2, %7, 0x80808080;\n\t"
      "addc.cc.u32 %3, %8, 0x80808080;\n\t"
      "addc.u32    %4, %9, 0x8080;"
      : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3), "=r"(r4)
      : "r"(y0), "r"(y1), "r"(y2), "r"(y3), "r"(y4));
  W[0] = r0;
  W[1] = r1;
  W[2] = r2;
  W[3] = r3;
  W[4] = r4 & 0xFFFFu;
#else
  uint64_t t = (uint64_t)0x80808080u + y0;
  W[0] = (uint32_t)t;
  t = (t >> 32) + 0x80808080u + y1;
  W[1] = (uint32_t)t;
  t = (t >> 32) + 0x80808080u + y2;
  W[2] = (uint32_t)t;
  t = (t >> 32) + 0x80808080u + y3;
  W[3] = (uint32_t)t;
  t = (t >> 32) + 0x8080u + y4;
  W[4] = (uint32_t)t & 0xFFFFu;
#endif
}

// The window for a chunk exponent E >= the element's lead exponent.
QB_HD void og_window(uint32_t w0, uint32_t w1, uint32_t w2, uint32_t w3, int E, uint32_t (&W)[5]) {
  og_window_s<false>(w0, w1, w2, w3, og_shift(E, w3), W);
}

// Digit t (0 = most significant) of an element with window W and sign bit
// neg: sign * (byte 17 - t of W, minus 128).
QB_HD int og_digit(const uint32_t (&W)[5], int t, uint32_t neg) {
  const int beta = 17 - t;
  const int d = (int)((W[beta >> 2] >> (8 * (beta & 3))) & 0xFFu) - 128;
  return neg ? -d : d;
}

// T = sum_{g<20} D_g 256^(19 - g) as six little-endian 32-bit words, two's
// complement: four diagonals at a time in 64-bit integers (|P| < 2^49),
// then T = P_0 2^128 + P_1 2^96 + P_2 2^64 + P_3 2^32 + P_4.
QB_HD void og_fold(const int32_t* D, uint32_t (&T)[6]) {
  int64_t P[5];
  for (int k = 0; k < 5; ++k) {
    int64_t p = D[4 * k];
    for (int i = 1; i < 4; ++i) p = p * 256 + D[4 * k + i];
    P[k] = p;
  }
  T[5] = (uint32_t)((uint64_t)P[0] >> 32);
  T[4] = (uint32_t)P[0];
  T[3] = T[2] = T[1] = T[0] = 0;
  // add P_k at words 4 - k and 5 - k (k = 1..4), sign-extended to word 5
  for (int k = 1; k < 5; ++k) {
    const int w = 4 - k;
    const uint32_t ext = 0u - (uint32_t)((uint64_t)P[k] >> 63);
    uint64_t c = (uint64_t)T[w] + (uint32_t)P[k];
    T[w] = (uint32_t)c;
    c = (c >> 32) + T[w + 1] + (uint32_t)((uint64_t)P[k] >> 32);
    T[w + 1] = (uint32_t)c;
    for (int i = w + 2; i < 6; ++i) {
      c = (c >> 32) + T[i] + ext;
      T[i] = (uint32_t)c;
    }
  }
}

// acc += T * 2^pe for a two's complement T of six words (|T| < 2^191).
QB_HD void og_wacc_add(wacc& acc, const uint32_t (&T)[6], int pe) {
  const uint32_t neg = T[5] >> 31, mask = 0u - neg;
  uint64_t c = (uint64_t)(T[0] ^ mask) + neg;
  const uint32_t a0 = (uint32_t)c;
  c = (c >> 32) + (T[1] ^ mask);
  const uint32_t a1 = (uint32_t)c;
  c = (c >> 32) + (T[2] ^ mask);
  const uint32_t a2 = (uint32_t)c;
  c = (c >> 32) + (T[3] ^ mask);
  const uint32_t a3 = (uint32_t)c;
  c = (c >> 32) + (T[4] ^ mask);
  const uint32_t a4 = (uint32_t)c;
  c = (c >> 32) + (T[5] ^ mask);
  const uint32_t a5 = (uint32_t)c;
  if ((a0 | a1 | a2 | a3 | a4 | a5) == 0) return;
  wacc_add_aligned(acc, a0, a1, a2, a3, a4, a5, 0u, pe, neg);
}

// Error budget of a row, in units of acc's least significant bit, for nch
// chunk additions (each drops less than one unit in its own alignment and
// one when it moves the frame up) with largest E + F = gmax, plus extra
// units (merges); coarsens acc when the Ozaki bound would not fit in 64 bits.
QB_HD uint64_t og_row_error(wacc& acc, uint32_t nch, int gmax, uint64_t extra) {
  uint64_t err = 2 * (uint64_t)nch + extra;
  int k = gmax - kOgErrShift - acc.e;
  if (k > 32) {
    const int c = k - 32;
    wacc_ashr(acc, c);
    acc.e += c;
    err = (c >= 64 ? 0 : (err >> c)) + 2;
    k = 32;
  }
  return err + (k <= 0 ? (uint64_t)nch : ((uint64_t)nch << k));
}

}  // namespace qb
