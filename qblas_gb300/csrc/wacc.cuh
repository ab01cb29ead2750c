// Wide fixed-point accumulator for binary128 dot products.
//
// The reference sums a dot product as a chain of correctly rounded FMAs
// (include/quadblas/algorithms/level1.hpp:14-35; level2.hpp:37-48;
// level3.hpp:77-85), so every term adds a rounding error of up to half an
// ulp of the running sum.  Here every product a_i*b_i is formed exactly
// (226-bit significand) and added into a 256-bit two's complement frame
// whose exponent floats with the largest product seen; the sum is rounded
// to binary128 once at the end.  The only approximations are that a product
// keeps its top 224 bits (relative error < 2^-222) and that bits shifted
// below the frame's least significant bit are dropped (at most one unit of
// 2^-192 of the largest product per term), so the result is the correctly
// rounded exact sum except when the exact sum lies within about
// n * 2^-190 * max|a_i b_i| of a rounding boundary.  This is far inside the
// required reduction bound k * u_q * sum|a_i b_i| (u_q = 2^-113).
//
// Compiled both for the device (PTX carry chains) and for the host (plain
// C++), with identical results.
#pragma once
#include "softquad.cuh"

namespace qb {

// Operand unpacked for multiplication: significand with its leading one at
// bit 127 of (m3:m2:m1:m0), value = m * 2^e, sign s.
// cls: 0 finite nonzero, 1 zero, 2 infinity, 3 NaN.
struct qop {
  uint32_t m0, m1, m2, m3;
  int32_t e;
  uint32_t s;
  uint32_t cls;
};

enum : uint32_t { kClsFinite = 0, kClsZero = 1, kClsInf = 2, kClsNan = 3 };

QB_HD uint32_t fshl32(uint32_t lo, uint32_t hi, uint32_t s) {  // ((hi:lo) << s) >> 32, 0 < s < 32
#if defined(__CUDA_ARCH__)
  return __funnelshift_l(lo, hi, s);
#else
  return (hi << s) | (lo >> (32 - s));
#endif
}

// Unpack a binary128 value.  Normal numbers take a few 32-bit funnel
// shifts; zero, subnormal, infinity and NaN take a branch.
QB_HD qop qop_unpack(q128 a) {
  qop r;
  const uint32_t w0 = (uint32_t)a.lo, w1 = (uint32_t)(a.lo >> 32);
  const uint32_t w2 = (uint32_t)a.hi, w3 = (uint32_t)(a.hi >> 32);
  const uint32_t be = (w3 >> 16) & 0x7fffu;
  r.s = w3 >> 31;
  if (be - 1u < 0x7ffeu) {  // normal: significand (hidden bit | 112 bits) << 15
    const uint32_t s3 = (w3 & 0xFFFFu) | 0x10000u;
    r.m3 = fshl32(w2, s3, 15);
    r.m2 = fshl32(w1, w2, 15);
    r.m1 = fshl32(w0, w1, 15);
    r.m0 = w0 << 15;
    r.e = (int)be - kBias - 127;
    r.cls = kClsFinite;
    return r;
  }
  uint64_t mh = a.hi & kMantHiMask, ml = a.lo;
  if (be == 0) {
    if ((mh | ml) == 0) {
      r.cls = kClsZero;
      r.m0 = r.m1 = r.m2 = r.m3 = 0;
      r.e = 0;
      return r;
    }
    int E;
    q_unpack_norm(a, mh, ml, E);
    uint64_t th = (mh << 15) | (ml >> 49);
    uint64_t tl = ml << 15;
    r.m0 = (uint32_t)tl;
    r.m1 = (uint32_t)(tl >> 32);
    r.m2 = (uint32_t)th;
    r.m3 = (uint32_t)(th >> 32);
    r.e = E - 127;
    r.cls = kClsFinite;
    return r;
  }
  r.cls = ((mh | ml) != 0) ? kClsNan : kClsInf;
  r.m0 = r.m1 = r.m2 = r.m3 = 0;
  r.e = 0;
  return r;
}

// Accumulator: value = W * 2^e with W a 256-bit two's complement integer
// (w0 least significant) plus special-value flags.
// Invariants: products are added with their top bit at frame bit <= 223;
// |W| < 2^255 holds for up to 2^31 added products.
struct wacc {
  uint32_t w0, w1, w2, w3, w4, w5, w6, w7;
  int32_t e;
  uint32_t flags;  // bit0 NaN, bit1 +inf, bit2 -inf
};

constexpr int32_t kWaccEmptyExp = -(1 << 30);

QB_HD void wacc_init(wacc& a) {
  a.w0 = a.w1 = a.w2 = a.w3 = a.w4 = a.w5 = a.w6 = a.w7 = 0;
  a.e = kWaccEmptyExp;
  a.flags = 0;
}

QB_HD uint32_t fshr32(uint32_t lo, uint32_t hi, uint32_t s) {  // ((hi:lo) >> s) mod 2^32, s < 32
#if defined(__CUDA_ARCH__)
  return __funnelshift_r(lo, hi, s);
#else
  return s ? (lo >> s) | (hi << (32 - s)) : lo;
#endif
}

// Arithmetic right shift of W by k >= 0 bits.
QB_HD void wacc_ashr(wacc& a, int k) {
  if (k <= 0) return;
  uint32_t fill = (uint32_t)((int32_t)a.w7 >> 31);
  if (k >= 256) {
    a.w0 = a.w1 = a.w2 = a.w3 = a.w4 = a.w5 = a.w6 = a.w7 = fill;
    return;
  }
  uint32_t b = (uint32_t)k & 31u;
  int w = k >> 5;
  uint32_t t0 = fshr32(a.w0, a.w1, b), t1 = fshr32(a.w1, a.w2, b), t2 = fshr32(a.w2, a.w3, b),
           t3 = fshr32(a.w3, a.w4, b), t4 = fshr32(a.w4, a.w5, b), t5 = fshr32(a.w5, a.w6, b),
           t6 = fshr32(a.w6, a.w7, b), t7 = fshr32(a.w7, fill, b);
  if (w & 4) {
    t0 = t4; t1 = t5; t2 = t6; t3 = t7;
    t4 = t5 = t6 = t7 = fill;
  }
  if (w & 2) {
    t0 = t2; t1 = t3; t2 = t4; t3 = t5; t4 = t6; t5 = t7;
    t6 = t7 = fill;
  }
  if (w & 1) {
    t0 = t1; t1 = t2; t2 = t3; t3 = t4; t4 = t5; t5 = t6; t6 = t7;
    t7 = fill;
  }
  a.w0 = t0; a.w1 = t1; a.w2 = t2; a.w3 = t3;
  a.w4 = t4; a.w5 = t5; a.w6 = t6; a.w7 = t7;
}

// 256-bit product of two 128-bit significands, returning limbs 1..7
// (the top 224 bits; limb 0 is dropped).
QB_HD void mul128x128_top224(const qop& a, const qop& b, uint32_t& p1, uint32_t& p2, uint32_t& p3,
                             uint32_t& p4, uint32_t& p5, uint32_t& p6, uint32_t& p7) {
#if defined(__CUDA_ARCH__)
  uint32_t r1, r2, r3, r4, r5, r6, r7;
  asm("{\n\t"
      // row 0 (limb 0, lo(a0*b0), is never needed: nothing carries out of it)
      "mul.lo.u32      %0, %7, %12;\n\t"
      "mul.lo.u32      %1, %7, %13;\n\t"
      "mul.lo.u32      %2, %7, %14;\n\t"
      "mad.hi.cc.u32   %0, %7, %11, %0;\n\t"
      "madc.hi.cc.u32  %1, %7, %12, %1;\n\t"
      "madc.hi.cc.u32  %2, %7, %13, %2;\n\t"
      "madc.hi.u32     %3, %7, %14, 0;\n\t"
      // row 1
      "mad.lo.cc.u32   %0, %8, %11, %0;\n\t"
      "madc.lo.cc.u32  %1, %8, %12, %1;\n\t"
      "madc.lo.cc.u32  %2, %8, %13, %2;\n\t"
      "madc.lo.cc.u32  %3, %8, %14, %3;\n\t"
      "addc.u32        %4, 0, 0;\n\t"
      "mad.hi.cc.u32   %1, %8, %11, %1;\n\t"
      "madc.hi.cc.u32  %2, %8, %12, %2;\n\t"
      "madc.hi.cc.u32  %3, %8, %13, %3;\n\t"
      "madc.hi.u32     %4, %8, %14, %4;\n\t"
      // row 2
      "mad.lo.cc.u32   %1, %9, %11, %1;\n\t"
      "madc.lo.cc.u32  %2, %9, %12, %2;\n\t"
      "madc.lo.cc.u32  %3, %9, %13, %3;\n\t"
      "madc.lo.cc.u32  %4, %9, %14, %4;\n\t"
      "addc.u32        %5, 0, 0;\n\t"
      "mad.hi.cc.u32   %2, %9, %11, %2;\n\t"
      "madc.hi.cc.u32  %3, %9, %12, %3;\n\t"
      "madc.hi.cc.u32  %4, %9, %13, %4;\n\t"
      "madc.hi.u32     %5, %9, %14, %5;\n\t"
      // row 3
      "mad.lo.cc.u32   %2, %10, %11, %2;\n\t"
      "madc.lo.cc.u32  %3, %10, %12, %3;\n\t"
      "madc.lo.cc.u32  %4, %10, %13, %4;\n\t"
      "madc.lo.cc.u32  %5, %10, %14, %5;\n\t"
      "addc.u32        %6, 0, 0;\n\t"
      "mad.hi.cc.u32   %3, %10, %11, %3;\n\t"
      "madc.hi.cc.u32  %4, %10, %12, %4;\n\t"
      "madc.hi.cc.u32  %5, %10, %13, %5;\n\t"
      "madc.hi.u32     %6, %10, %14, %6;\n\t"
      "}"
      : "=&r"(r1), "=&r"(r2), "=&r"(r3), "=&r"(r4), "=&r"(r5), "=&r"(r6), "=&r"(r7)
      : "r"(a.m0), "r"(a.m1), "r"(a.m2), "r"(a.m3), "r"(b.m0), "r"(b.m1), "r"(b.m2), "r"(b.m3));
  p1 = r1; p2 = r2; p3 = r3; p4 = r4; p5 = r5; p6 = r6; p7 = r7;
#else
  uint32_t A[4] = {a.m0, a.m1, a.m2, a.m3}, B[4] = {b.m0, b.m1, b.m2, b.m3};
  uint32_t r[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = 0; i < 4; ++i) {
    uint64_t c = 0;
    for (int j = 0; j < 4; ++j) {
      uint64_t t = (uint64_t)A[i] * B[j] + r[i + j] + c;
      r[i + j] = (uint32_t)t;
      c = t >> 32;
    }
    r[i + 4] = (uint32_t)c;
  }
  p1 = r[1]; p2 = r[2]; p3 = r[3]; p4 = r[4]; p5 = r[5]; p6 = r[6]; p7 = r[7];
#endif
}

// Limbs 2..7 of the 256-bit product of two 128-bit significands, without
// the partial products that feed only limbs 0 and 1 (lo(a0 b0), hi(a0 b0),
// lo(a0 b1), lo(a1 b0)) and their carries: the result is below the exact
// top 192 bits by less than 4, i.e. less than 2^34 units of limb 1.  Three
// multiplies fewer than mul128x128_top224.
QB_HD void mul128x128_top192(const qop& a, const qop& b, uint32_t& p2, uint32_t& p3, uint32_t& p4,
                             uint32_t& p5, uint32_t& p6, uint32_t& p7) {
#if defined(__CUDA_ARCH__)
  uint32_t r2, r3, r4, r5, r6, r7;
  asm("{\n\t"
      // row 0: lo(a0 b2), lo(a0 b3); hi(a0 b1), hi(a0 b2), hi(a0 b3)
      "mul.lo.u32      %0, %6, %12;\n\t"
      "mul.lo.u32      %1, %6, %13;\n\t"
      "mad.hi.cc.u32   %0, %6, %11, %0;\n\t"
      "madc.hi.cc.u32  %1, %6, %12, %1;\n\t"
      "madc.hi.u32     %2, %6, %13, 0;\n\t"
      // row 1: lo(a1 b1..b3) into limbs 2..4, hi(a1 b0..b3) into limbs 2..5
      "mad.lo.cc.u32   %0, %7, %11, %0;\n\t"
      "madc.lo.cc.u32  %1, %7, %12, %1;\n\t"
      "madc.lo.cc.u32  %2, %7, %13, %2;\n\t"
      "addc.u32        %3, 0, 0;\n\t"
      "mad.hi.cc.u32   %0, %7, %10, %0;\n\t"
      "madc.hi.cc.u32  %1, %7, %11, %1;\n\t"
      "madc.hi.cc.u32  %2, %7, %12, %2;\n\t"
      "madc.hi.u32     %3, %7, %13, %3;\n\t"
      // row 2: lo(a2 b0..b3) into limbs 2..5, hi into limbs 3..6
      "mad.lo.cc.u32   %0, %8, %10, %0;\n\t"
      "madc.lo.cc.u32  %1, %8, %11, %1;\n\t"
      "madc.lo.cc.u32  %2, %8, %12, %2;\n\t"
      "madc.lo.cc.u32  %3, %8, %13, %3;\n\t"
      "addc.u32        %4, 0, 0;\n\t"
      "mad.hi.cc.u32   %1, %8, %10, %1;\n\t"
      "madc.hi.cc.u32  %2, %8, %11, %2;\n\t"
      "madc.hi.cc.u32  %3, %8, %12, %3;\n\t"
      "madc.hi.u32     %4, %8, %13, %4;\n\t"
      // row 3: lo(a3 b0..b3) into limbs 3..6, hi into limbs 4..7
      "mad.lo.cc.u32   %1, %9, %10, %1;\n\t"
      "madc.lo.cc.u32  %2, %9, %11, %2;\n\t"
      "madc.lo.cc.u32  %3, %9, %12, %3;\n\t"
      "madc.lo.cc.u32  %4, %9, %13, %4;\n\t"
      "addc.u32        %5, 0, 0;\n\t"
      "mad.hi.cc.u32   %2, %9, %10, %2;\n\t"
      "madc.hi.cc.u32  %3, %9, %11, %3;\n\t"
      "madc.hi.cc.u32  %4, %9, %12, %4;\n\t"
      "madc.hi.u32     %5, %9, %13, %5;\n\t"
      "}"
      : "=&r"(r2), "=&r"(r3), "=&r"(r4), "=&r"(r5), "=&r"(r6), "=&r"(r7)
      : "r"(a.m0), "r"(a.m1), "r"(a.m2), "r"(a.m3), "r"(b.m0), "r"(b.m1), "r"(b.m2), "r"(b.m3));
  p2 = r2; p3 = r3; p4 = r4; p5 = r5; p6 = r6; p7 = r7;
#else
  uint32_t A[4] = {a.m0, a.m1, a.m2, a.m3}, B[4] = {b.m0, b.m1, b.m2, b.m3};
  uint32_t r[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  // lo(a_i b_j) belongs to limb i + j, hi(a_i b_j) to limb i + j + 1; the
  // halves in limbs 0 and 1 are dropped, the rest summed column by column
  uint64_t col[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      const uint64_t prod = (uint64_t)A[i] * B[j];
      if (i + j >= 2) col[i + j] += (uint32_t)prod;
      if (i + j + 1 >= 2) col[i + j + 1] += prod >> 32;
    }
  uint64_t c = 0;
  for (int k = 2; k < 8; ++k) {
    const uint64_t t = col[k] + c;
    r[k] = (uint32_t)t;
    c = t >> 32;
  }
  p2 = r[2]; p3 = r[3]; p4 = r[4]; p5 = r[5]; p6 = r[6]; p7 = r[7];
#endif
}

// W += (neg ? -Q : Q) for a 256-bit Q = (q7..q0).
QB_HD void wacc_add_signed(wacc& a, uint32_t q0, uint32_t q1, uint32_t q2, uint32_t q3, uint32_t q4,
                           uint32_t q5, uint32_t q6, uint32_t q7, uint32_t neg) {
  uint32_t mask = 0u - neg;
  q0 ^= mask; q1 ^= mask; q2 ^= mask; q3 ^= mask;
  q4 ^= mask; q5 ^= mask; q6 ^= mask; q7 ^= mask;
#if defined(__CUDA_ARCH__)
  asm("{\n\t"
      ".reg .u32 t;\n\t"
      "add.cc.u32  t, %16, %16;\n\t"  // carry-in = neg (mask + mask overflows iff mask != 0)
      "addc.cc.u32 %0, %0, %8;\n\t"
      "addc.cc.u32 %1, %1, %9;\n\t"
      "addc.cc.u32 %2, %2, %10;\n\t"
      "addc.cc.u32 %3, %3, %11;\n\t"
      "addc.cc.u32 %4, %4, %12;\n\t"
      "addc.cc.u32 %5, %5, %13;\n\t"
      "addc.cc.u32 %6, %6, %14;\n\t"
      "addc.u32    %7, %7, %15;\n\t"
      "}"
      : "+r"(a.w0), "+r"(a.w1), "+r"(a.w2), "+r"(a.w3), "+r"(a.w4), "+r"(a.w5), "+r"(a.w6),
        "+r"(a.w7)
      : "r"(q0), "r"(q1), "r"(q2), "r"(q3), "r"(q4), "r"(q5), "r"(q6), "r"(q7), "r"(mask));
#else
  uint64_t c = neg;
  uint32_t* w[8] = {&a.w0, &a.w1, &a.w2, &a.w3, &a.w4, &a.w5, &a.w6, &a.w7};
  uint32_t q[8] = {q0, q1, q2, q3, q4, q5, q6, q7};
  for (int i = 0; i < 8; ++i) {
    uint64_t t = (uint64_t)*w[i] + q[i] + c;
    *w[i] = (uint32_t)t;
    c = t >> 32;
  }
#endif
}

// Flags for a product of two operands of which at least one is not finite
// nonzero, or 0 when the product is an exact zero.
QB_HD uint32_t special_product_flags(const qop& a, const qop& b) {
  if (a.cls == kClsNan || b.cls == kClsNan) return 1u;
  bool ia = a.cls == kClsInf, ib = b.cls == kClsInf;
  if (ia || ib) {
    if (a.cls == kClsZero || b.cls == kClsZero) return 1u;  // inf * 0
    return (a.s ^ b.s) ? 4u : 2u;
  }
  return 0u;
}

// acc += (neg ? -P : P) * 2^pe for a magnitude P = (p7..p1) < 2^224: P is
// aligned to the frame (moving the frame up when P's least significant bit
// lies above it), dropping less than one unit of the frame's last bit.
QB_HD void wacc_add_aligned(wacc& acc, uint32_t p1, uint32_t p2, uint32_t p3, uint32_t p4, uint32_t p5,
                            uint32_t p6, uint32_t p7, int pe, uint32_t neg) {
  int r = acc.e - pe;       // right shift that aligns P to the frame
  if (r < 0) {              // product above the frame top: move the frame up
    wacc_ashr(acc, -r);
    acc.e = pe;
    r = 0;
  }
  uint32_t q0, q1, q2, q3, q4, q5, q6;
  if (r >= 224) return;  // entirely below the frame
  uint32_t b5 = (uint32_t)r & 31u;
  q0 = fshr32(p1, p2, b5);
  q1 = fshr32(p2, p3, b5);
  q2 = fshr32(p3, p4, b5);
  q3 = fshr32(p4, p5, b5);
  q4 = fshr32(p5, p6, b5);
  q5 = fshr32(p6, p7, b5);
  q6 = fshr32(p7, 0u, b5);
  int w = r >> 5;
  if (w & 4) {
    q0 = q4; q1 = q5; q2 = q6;
    q3 = q4 = q5 = q6 = 0;
  }
  if (w & 2) {
    q0 = q2; q1 = q3; q2 = q4; q3 = q5; q4 = q6;
    q5 = q6 = 0;
  }
  if (w & 1) {
    q0 = q1; q1 = q2; q2 = q3; q3 = q4; q4 = q5; q5 = q6;
    q6 = 0;
  }
  wacc_add_signed(acc, q0, q1, q2, q3, q4, q5, q6, 0u, neg);
}

// acc += a * b
QB_HD void wacc_add_product(wacc& acc, const qop& a, const qop& b) {
  if ((a.cls | b.cls) != kClsFinite) {
    acc.flags |= special_product_flags(a, b);
    return;
  }
  uint32_t p1, p2, p3, p4, p5, p6, p7;
  mul128x128_top224(a, b, p1, p2, p3, p4, p5, p6, p7);
  wacc_add_aligned(acc, p1, p2, p3, p4, p5, p6, p7, a.e + b.e + 32, a.s ^ b.s);
}

// acc += a * b with mul128x128_top192: each product adds less than 2^34 + 2
// units of the frame's last bit to the error (instead of 2).
QB_HD void wacc_add_product_trunc(wacc& acc, const qop& a, const qop& b) {
  if ((a.cls | b.cls) != kClsFinite) {
    acc.flags |= special_product_flags(a, b);
    return;
  }
  uint32_t p2, p3, p4, p5, p6, p7;
  mul128x128_top192(a, b, p2, p3, p4, p5, p6, p7);
  wacc_add_aligned(acc, 0u, p2, p3, p4, p5, p6, p7, a.e + b.e + 32, a.s ^ b.s);
}

// a += b (b unchanged).  The smaller-exponent operand is aligned to the larger one's frame.  The
// frame moves up one bit only when an operand could make the sum overflow
// (|W| >= 2^254, seen as the top two bits differing), so a chain of merges
// drops no low-order bits unless the magnitude really grows.
QB_HD void wacc_merge(wacc& a, const wacc& b) {
  a.flags |= b.flags;
  wacc t = b;
  if (a.e < t.e) {
    wacc u = a;
    a = t;
    a.flags = u.flags;
    t = u;
  }
  wacc_ashr(t, a.e - t.e);
  const uint32_t big = ((a.w7 ^ (a.w7 << 1)) | (t.w7 ^ (t.w7 << 1))) >> 31;
  if (big) {
    wacc_ashr(a, 1);
    wacc_ashr(t, 1);
    a.e += 1;
  }
  wacc_add_signed(a, t.w0, t.w1, t.w2, t.w3, t.w4, t.w5, t.w6, t.w7, 0u);
}

// Round the accumulated value to binary128.
QB_HD q128 wacc_round(const wacc& a) {
  if ((a.flags & 1u) || ((a.flags & 6u) == 6u)) return q_nan();
  if (a.flags & 2u) return q_inf(0);
  if (a.flags & 4u) return q_inf(1);
  uint32_t neg = a.w7 >> 31;
  uint32_t mask = 0u - neg;
  // magnitude = neg ? -W : W
  uint64_t x0 = ((uint64_t)(a.w1 ^ mask) << 32) | (a.w0 ^ mask);
  uint64_t x1 = ((uint64_t)(a.w3 ^ mask) << 32) | (a.w2 ^ mask);
  uint64_t x2 = ((uint64_t)(a.w5 ^ mask) << 32) | (a.w4 ^ mask);
  uint64_t x3 = ((uint64_t)(a.w7 ^ mask) << 32) | (a.w6 ^ mask);
  u256 M = u256_make(x3, x2, x1, x0);
  if (neg) M = u256_add(M, u256_make(0, 0, 0, 1));
  return round_pack(neg, M, false, a.e);
}

}  // namespace qb
