// ORACLE — test infrastructure only; never linked into the product.
//
// Stand-in for SLEEF 3.8's <sleefquad.h> (the reference pins SLEEF 3.8 in
// .github/workflows/ci.yml:26; SLEEF itself is not vendored in the
// reference and is not installed here).  It supplies exactly the symbols the
// reference headers call (include/quadblas/core/platform.hpp:19,
// include/quadblas/simd/quad_vector.hpp:28-146, the algorithms and the C
// interface) on top of the compiler's IEEE binary128 type:
//   x86-64  : GCC __float128 with libquadmath fmaq/sqrtq
//   aarch64 : long double (IEEE binary128 under the AAPCS64) with fmal/sqrtl
// Both are correctly rounded (RNE), which is what SLEEF's *_u05 functions
// document (<= 0.5000000001 ulp), so results agree with SLEEF bit for bit
// except possibly in NaN payloads.
#ifndef QBLAS_ORACLE_SLEEF_SHIM_H
#define QBLAS_ORACLE_SLEEF_SHIM_H

#if defined(__x86_64__)
#include <quadmath.h>
typedef __float128 Sleef_quad;
#define QSHIM_FMA fmaq
#define QSHIM_SQRT sqrtq
#elif defined(__aarch64__)
#include <math.h>
typedef long double Sleef_quad;
#define QSHIM_FMA fmal
#define QSHIM_SQRT sqrtl
#else
#error "binary128 shim: unsupported host"
#endif

typedef struct {
  Sleef_quad v[2];
} Sleef_quadx2;

static inline Sleef_quad Sleef_addq1_u05(Sleef_quad a, Sleef_quad b) { return a + b; }
static inline Sleef_quad Sleef_mulq1_u05(Sleef_quad a, Sleef_quad b) { return a * b; }
static inline Sleef_quad Sleef_fmaq1_u05(Sleef_quad a, Sleef_quad b, Sleef_quad c) {
  return QSHIM_FMA(a, b, c);
}
static inline Sleef_quad Sleef_sqrtq1_u05(Sleef_quad a) { return QSHIM_SQRT(a); }
static inline Sleef_quad Sleef_cast_from_doubleq1(double d) { return (Sleef_quad)d; }
static inline double Sleef_cast_to_doubleq1(Sleef_quad q) { return (double)q; }

#define QSHIM_X2(SUFFIX)                                                                  \
  static inline Sleef_quadx2 Sleef_splatq2_##SUFFIX(Sleef_quad a) {                       \
    Sleef_quadx2 r;                                                                       \
    r.v[0] = a;                                                                           \
    r.v[1] = a;                                                                           \
    return r;                                                                             \
  }                                                                                       \
  static inline Sleef_quadx2 Sleef_loadq2_##SUFFIX(Sleef_quad* p) {                       \
    Sleef_quadx2 r;                                                                       \
    r.v[0] = p[0];                                                                        \
    r.v[1] = p[1];                                                                        \
    return r;                                                                             \
  }                                                                                       \
  static inline Sleef_quad Sleef_getq2_##SUFFIX(Sleef_quadx2 x, int i) { return x.v[i]; } \
  static inline Sleef_quadx2 Sleef_addq2_u05##SUFFIX(Sleef_quadx2 a, Sleef_quadx2 b) {    \
    Sleef_quadx2 r;                                                                       \
    r.v[0] = a.v[0] + b.v[0];                                                             \
    r.v[1] = a.v[1] + b.v[1];                                                             \
    return r;                                                                             \
  }                                                                                       \
  static inline Sleef_quadx2 Sleef_mulq2_u05##SUFFIX(Sleef_quadx2 a, Sleef_quadx2 b) {    \
    Sleef_quadx2 r;                                                                       \
    r.v[0] = a.v[0] * b.v[0];                                                             \
    r.v[1] = a.v[1] * b.v[1];                                                             \
    return r;                                                                             \
  }                                                                                       \
  static inline Sleef_quadx2 Sleef_fmaq2_u05##SUFFIX(Sleef_quadx2 a, Sleef_quadx2 b,      \
                                                     Sleef_quadx2 c) {                    \
    Sleef_quadx2 r;                                                                       \
    r.v[0] = QSHIM_FMA(a.v[0], b.v[0], c.v[0]);                                           \
    r.v[1] = QSHIM_FMA(a.v[1], b.v[1], c.v[1]);                                           \
    return r;                                                                             \
  }

QSHIM_X2(sse2)
QSHIM_X2(advsimd)

#endif
