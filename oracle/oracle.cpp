// ORACLE — test infrastructure only.  Only tests/, __graft_entry__.smoke()
// and the cpu_baseline / --impl reference legs of bench.py may load this
// library, and only as the checker or as the timed CPU baseline; the
// product (qblas_gb300) never links, loads or calls it.
//
// A CPU restatement of QuadBLAS's binary128 hot path in plain C++ on the
// host compiler's IEEE binary128 type (x86-64: __float128 + libquadmath;
// aarch64: long double + libm), plus an exact long accumulator.
//
//  1. Reference-order restatement (oq_ref_*): the same sequence of
//     correctly rounded operations as the reference, so its results are
//     bit-identical to the reference compiled through the SLEEF shim
//     (checked by tests against oracle/_ref and tests/golden fixtures).
//       dot   : include/quadblas/algorithms/level1.hpp:14-137
//       axpy  : include/quadblas/algorithms/level1.hpp:140-223
//       gemv  : include/quadblas/algorithms/level2.hpp:15-100
//       gemm  : include/quadblas/algorithms/level3.hpp:187-336 and the
//               k-panel size from include/quadblas/detail/blocking.hpp:17-66
//     plus the "test-file" semantics of test_quadblas.cpp:144-191
//     (one sequential FMA chain per output, layout-aware indexing), which
//     are the intended semantics for column-major and transposed calls.
//  2. Exact oracle (oq_exact_*): a Kulisch-style fixed-point accumulator
//     spanning the whole binary128 product range (2^-33212 .. 2^32832), so
//     sum_i x_i*y_i is held exactly and rounded once (RNE).  It also returns
//     the residual r = round(S - R), which measures any result in ulps of
//     the exact value S.
#include <float.h>
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#if defined(__x86_64__)
#include <quadmath.h>
typedef __float128 oq;
static inline oq q_fma(oq a, oq b, oq c) { return fmaq(a, b, c); }
static inline oq q_sqrt(oq a) { return sqrtq(a); }
static inline oq q_ldexp(oq a, int e) { return ldexpq(a, e); }
static inline oq q_fabs(oq a) { return fabsq(a); }
static inline int q_isnan(oq a) { return isnanq(a); }
static inline int q_isinf(oq a) { return isinfq(a); }
#elif defined(__aarch64__)
typedef long double oq;
static_assert(LDBL_MANT_DIG == 113, "long double must be IEEE binary128");
static inline oq q_fma(oq a, oq b, oq c) { return fmal(a, b, c); }
static inline oq q_sqrt(oq a) { return sqrtl(a); }
static inline oq q_ldexp(oq a, int e) { return ldexpl(a, e); }
static inline oq q_fabs(oq a) { return fabsl(a); }
static inline int q_isnan(oq a) { return isnan(a); }
static inline int q_isinf(oq a) { return isinf(a); }
#else
#error "oracle: unsupported host"
#endif
static_assert(sizeof(oq) == 16, "binary128 must be 16 bytes");

typedef unsigned __int128 u128;

// ---------------------------------------------------------------------------
// Bit-level access
// ---------------------------------------------------------------------------
static inline void q_bits(oq v, uint64_t& lo, uint64_t& hi) {
  uint64_t w[2];
  memcpy(w, &v, 16);
  lo = w[0];
  hi = w[1];
}
static inline oq q_from_bits(uint64_t lo, uint64_t hi) {
  uint64_t w[2] = {lo, hi};
  oq v;
  memcpy(&v, w, 16);
  return v;
}

static inline bool q_signbit(oq v) {
  uint64_t lo, hi;
  q_bits(v, lo, hi);
  return (hi >> 63) != 0;
}

// Finite nonzero value -> significand m (bit 112 set) and E with
// value = m * 2^(E-112).
static inline void q_unpack(oq v, u128& m, int& E) {
  uint64_t lo, hi;
  q_bits(v, lo, hi);
  int be = (int)((hi >> 48) & 0x7fff);
  m = ((u128)(hi & 0x0000FFFFFFFFFFFFull) << 64) | lo;
  if (be) {
    m |= (u128)1 << 112;
    E = be - 16383;
    return;
  }
  int sh = 0;
  while (!((m >> 112) & 1)) {
    m <<= 1;
    ++sh;
  }
  E = -16382 - sh;
}

// ---------------------------------------------------------------------------
// Elementwise (correctly rounded by the host libraries)
// ---------------------------------------------------------------------------
extern "C" {

void oq_fma_n(int64_t n, const oq* a, const oq* b, const oq* c, oq* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = q_fma(a[i], b[i], c[i]);
}
void oq_mul_n(int64_t n, const oq* a, const oq* b, oq* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = a[i] * b[i];
}
void oq_add_n(int64_t n, const oq* a, const oq* b, oq* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = a[i] + b[i];
}
void oq_sub_n(int64_t n, const oq* a, const oq* b, oq* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = a[i] - b[i];
}
void oq_sqrt_n(int64_t n, const oq* a, oq* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = q_sqrt(a[i]);
}
void oq_from_double_n(int64_t n, const double* d, oq* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = (oq)d[i];
}
void oq_to_double_n(int64_t n, const oq* a, double* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = (double)a[i];
}

// ---------------------------------------------------------------------------
// 1. Reference-order restatement
// ---------------------------------------------------------------------------

// level1.hpp:14-35 (dot_kernel_vectorized): two interleaved FMA lanes over
// pairs, lane sum by one correctly rounded add (quad_vector.hpp:141), then
// a scalar FMA tail.
static oq ref_dot_kernel(const oq* x, const oq* y, size_t n) {
  size_t vec_n = n / 2;
  oq s0 = 0, s1 = 0;
  for (size_t i = 0; i < vec_n; ++i) {
    s0 = q_fma(x[2 * i], y[2 * i], s0);
    s1 = q_fma(x[2 * i + 1], y[2 * i + 1], s1);
  }
  oq r = s0 + s1;
  for (size_t i = vec_n * 2; i < n; ++i) r = q_fma(x[i], y[i], r);
  return r;
}

static const size_t kParallelThreshold = 500;  // core/constants.hpp:14

// level1.hpp:38-137 (dot_parallel / dot) with T OpenMP threads.
void oq_ref_dot(int64_t n_, const oq* x, int64_t incx, const oq* y, int64_t incy, int nthreads,
                oq* out) {
  size_t n = (size_t)n_;
  if (n == 0) {
    *out = 0;
    return;
  }
  int T = nthreads < 1 ? 1 : nthreads;
  std::vector<oq> part(T, (oq)0);
  if (incx == 1 && incy == 1) {
    if (n < kParallelThreshold) {
      *out = ref_dot_kernel(x, y, n);
      return;
    }
    size_t chunk = n / T;
#pragma omp parallel for num_threads(T) schedule(static, 1)
    for (int t = 0; t < T; ++t) {
      size_t start = t * chunk;
      size_t end = (t == T - 1) ? n : start + chunk;
      if (start < end) part[t] = ref_dot_kernel(&x[start], &y[start], end - start);
    }
  } else {
    if (n < kParallelThreshold) {
      oq r = 0;
      for (size_t i = 0; i < n; ++i) r = q_fma(x[i * incx], y[i * incy], r);
      *out = r;
      return;
    }
    size_t chunk = n / T;
#pragma omp parallel for num_threads(T) schedule(static, 1)
    for (int t = 0; t < T; ++t) {
      size_t start = t * chunk;
      size_t end = (t == T - 1) ? n : start + chunk;
      oq r = 0;
      for (size_t i = start; i < end; ++i) r = q_fma(x[i * incx], y[i * incy], r);
      part[t] = r;
    }
  }
  oq r = 0;
  for (int t = 0; t < T; ++t) r = r + part[t];
  *out = r;
}

// level1.hpp:140-223 (axpy): y_i = fma(alpha, x_i, y_i), one rounding each.
void oq_ref_axpy(int64_t n, const oq* alpha, const oq* x, int64_t incx, oq* y, int64_t incy,
                 int nthreads) {
  oq a = *alpha;
#pragma omp parallel for num_threads(nthreads < 1 ? 1 : nthreads) schedule(static)
  for (int64_t i = 0; i < n; ++i) y[i * incy] = q_fma(x[i * incx], a, y[i * incy]);
}

// gemv.  lib_order = 1: the library order of level2.hpp:15-100 (row-major
// rows via the two-lane dot kernel when incx == 1; column-major as
// y *= beta then per-column y_i = fma(A_ij, alpha*x_j, y_i)).
// lib_order = 0: test_quadblas.cpp:162-173 (one FMA chain per row of A,
// then y_i = fma(alpha, sum, beta*y_i), for both layouts).
void oq_ref_gemv(int col_major, int64_t m, int64_t n, const oq* alpha, const oq* A, int64_t lda,
                 const oq* x, int64_t incx, const oq* beta, oq* y, int64_t incy, int lib_order,
                 int nthreads) {
  oq al = *alpha, be = *beta;
  int T = nthreads < 1 ? 1 : nthreads;
  if (m == 0 || n == 0) return;
  if (lib_order && col_major) {
    for (int64_t i = 0; i < m; ++i) y[i * incy] = be * y[i * incy];
    for (int64_t j = 0; j < n; ++j) {
      oq xj = al * x[j * incx];
      const oq* col = &A[j * lda];
#pragma omp parallel for num_threads(T) schedule(static)
      for (int64_t i = 0; i < m; ++i) y[i * incy] = q_fma(col[i], xj, y[i * incy]);
    }
    return;
  }
#pragma omp parallel for num_threads(T) schedule(static)
  for (int64_t i = 0; i < m; ++i) {
    oq sum = 0;
    if (lib_order && incx == 1) {
      sum = ref_dot_kernel(&A[i * lda], x, (size_t)n);
    } else {
      for (int64_t j = 0; j < n; ++j) {
        int64_t a_idx = col_major ? j * lda + i : i * lda + j;
        sum = q_fma(A[a_idx], x[j * incx], sum);
      }
    }
    y[i * incy] = q_fma(al, sum, be * y[i * incy]);
  }
}

// gemm.  lib_order = 1: level3.hpp:215-336 for row-major storage: when
// m, n, k <= 64 one FMA chain per element (gemm_simple, :187-213); else the
// k dimension is cut into panels of kc = max(min(126, k), 4) (the value
// BlockingParams computes on non-Apple hosts, blocking.hpp:17-66), each
// panel sum is an FMA chain from +0 and is folded into C as
// C = fma(alpha, panel_sum, beta_eff * C) with beta_eff = beta on the first
// panel and 1 afterwards (:299, :107).  lib_order = 0: test_quadblas.cpp
// :176-191 (one chain over all k, layout-aware indexing).
void oq_ref_gemm(int col_major, int64_t m, int64_t n, int64_t k, const oq* alpha, const oq* A,
                 int64_t lda, const oq* B, int64_t ldb, const oq* beta, oq* C, int64_t ldc,
                 int lib_order, int nthreads) {
  if (m == 0 || n == 0 || k == 0) return;
  oq al = *alpha, be = *beta;
  int64_t kc = k;
  if (lib_order && !(m <= 64 && n <= 64 && k <= 64)) {
    kc = std::max<int64_t>(std::min<int64_t>(126, k), 4);
  }
  int T = nthreads < 1 ? 1 : nthreads;
#pragma omp parallel for collapse(2) num_threads(T) schedule(static)
  for (int64_t i = 0; i < m; ++i) {
    for (int64_t j = 0; j < n; ++j) {
      int64_t c_idx = col_major ? j * ldc + i : i * ldc + j;
      oq c = C[c_idx];
      for (int64_t kk = 0; kk < k; kk += kc) {
        int64_t ke = std::min(k, kk + kc);
        oq sum = 0;
        for (int64_t l = kk; l < ke; ++l) {
          int64_t a_idx = col_major ? l * lda + i : i * lda + l;
          int64_t b_idx = col_major ? j * ldb + l : l * ldb + j;
          sum = q_fma(A[a_idx], B[b_idx], sum);
        }
        oq bc = (kk == 0) ? be * c : c;
        c = q_fma(al, sum, bc);
      }
      C[c_idx] = c;
    }
  }
}

// ---------------------------------------------------------------------------
// 2. Exact long accumulator
// ---------------------------------------------------------------------------
// value = sum_i D[i] * 2^(32*i - kOffset), D[i] int64 carry-save digits.
static const int kOffset = 33216;          // bit position of 2^0
static const int kDigits = 33216 / 32 + 1024 + 16;

struct LongAcc {
  int64_t D[kDigits];
  int lo, hi;       // touched digit range
  int64_t nadds;
  bool nan, pinf, ninf;
  void clear() {
    if (hi >= lo) memset(&D[lo], 0, sizeof(int64_t) * (hi - lo + 1));
    lo = kDigits;
    hi = -1;
    nadds = 0;
    nan = pinf = ninf = false;
  }
  LongAcc() {
    memset(D, 0, sizeof(D));
    lo = kDigits;
    hi = -1;
    nadds = 0;
    nan = pinf = ninf = false;
  }
  // Carry-propagates the digits into [0, 2^32), except that a negative
  // total keeps its sign in a negative top digit: value =
  // sum_{i<hi} D_i 2^(32 i) + D_hi 2^(32 hi) with D_hi in [-2^32, 0).
  // Idempotent: repeated calls do not grow the digit range.
  void normalize() {
    if (hi < lo) return;
    int64_t carry = 0;
    for (int i = lo; i <= hi; ++i) {
      int64_t v = D[i] + carry;
      D[i] = v & 0xffffffffLL;
      carry = v >> 32;  // arithmetic
    }
    while (carry != 0 && carry != -1) {
      ++hi;
      int64_t v = D[hi] + carry;
      D[hi] = v & 0xffffffffLL;
      carry = v >> 32;
    }
    if (carry == -1) {
      // value = digits - 2^(32(hi+1)): drop all-ones sign-extension digits,
      // then fold the borrow into the top digit
      while (hi > lo && D[hi] == 0xffffffffLL) {
        D[hi] = 0;
        --hi;
      }
      D[hi] -= (1LL << 32);
    }
    nadds = 0;
  }
  // add sign * P * 2^(bitpos - kOffset) where P < 2^256 (four 64-bit words)
  void add_mag(const uint64_t P[4], int bitpos, bool neg) {
    int w = bitpos >> 5, b = bitpos & 31;
    uint32_t piece[9];
    uint64_t ext[5] = {P[0], P[1], P[2], P[3], 0};
    for (int k = 0; k < 9; ++k) {
      // bits [32k - b, 32k - b + 32) of P
      int bit = 32 * k - b;
      uint64_t v;
      if (bit < 0) {
        v = (ext[0] << (-bit));
      } else {
        int wi = bit >> 6, wb = bit & 63;
        v = ext[wi] >> wb;
        if (wb > 32 && wi + 1 < 5) v |= ext[wi + 1] << (64 - wb);
      }
      piece[k] = (uint32_t)v;
    }
    for (int k = 0; k < 9; ++k) {
      if (!piece[k]) continue;
      int d = w + k;
      D[d] += neg ? -(int64_t)piece[k] : (int64_t)piece[k];
      if (d < lo) lo = d;
      if (d > hi) hi = d;
    }
    if (++nadds >= (1LL << 29)) normalize();
  }
  void add_product(oq a, oq b) {
    if (q_isnan(a) || q_isnan(b)) {
      nan = true;
      return;
    }
    bool neg = q_signbit(a) != q_signbit(b);
    if (q_isinf(a) || q_isinf(b)) {
      if (a == 0 || b == 0) {
        nan = true;
        return;
      }
      (neg ? ninf : pinf) = true;
      return;
    }
    if (a == 0 || b == 0) return;
    u128 ma, mb;
    int Ea, Eb;
    q_unpack(a, ma, Ea);
    q_unpack(b, mb, Eb);
    uint64_t al = (uint64_t)ma, ah = (uint64_t)(ma >> 64);
    uint64_t bl = (uint64_t)mb, bh = (uint64_t)(mb >> 64);
    u128 p0 = (u128)al * bl, p1 = (u128)al * bh, p2 = (u128)ah * bl, p3 = (u128)ah * bh;
    // sum into 256 bits
    u128 mid = (p0 >> 64) + (uint64_t)p1 + (uint64_t)p2;
    uint64_t w0 = (uint64_t)p0, w1 = (uint64_t)mid;
    u128 hi2 = (mid >> 64) + (p1 >> 64) + (p2 >> 64) + (uint64_t)p3;
    uint64_t w2 = (uint64_t)hi2;
    uint64_t w3 = (uint64_t)((hi2 >> 64) + (p3 >> 64));
    uint64_t P[4] = {w0, w1, w2, w3};
    int Ep = Ea + Eb - 224;
    add_mag(P, Ep + kOffset, neg);
  }
  void add_value(oq c, bool negate) {
    if (q_isnan(c)) {
      nan = true;
      return;
    }
    bool neg = q_signbit(c) != negate;
    if (q_isinf(c)) {
      (neg ? ninf : pinf) = true;
      return;
    }
    if (c == 0) return;
    u128 m;
    int E;
    q_unpack(c, m, E);
    uint64_t P[4] = {(uint64_t)m, (uint64_t)(m >> 64), 0, 0};
    add_mag(P, E - 112 + kOffset, neg);
  }
  // Round the exact value to binary128 (RNE).  Normalizes in place.
  oq round() {
    if (nan || (pinf && ninf)) return (oq)NAN;
    if (pinf) return (oq)INFINITY;
    if (ninf) return -(oq)INFINITY;
    normalize();
    if (hi < lo) return 0;
    bool neg = D[hi] < 0;
    // magnitude digits (one spare digit above hi for the negation)
    int n = hi - lo + 2;
    std::vector<uint32_t> mag(n, 0u);
    if (!neg) {
      for (int i = 0; i + 1 < n; ++i) mag[i] = (uint32_t)D[lo + i];
    } else {
      // two's complement negation of digits lo..hi, sign-extended by one digit
      uint64_t carry = 1;
      for (int i = 0; i < n; ++i) {
        uint32_t d = i + 1 < n ? (uint32_t)D[lo + i] : 0xffffffffu;
        uint64_t v = (uint64_t)(uint32_t)(~d) + carry;
        mag[i] = (uint32_t)v;
        carry = v >> 32;
      }
    }
    int top = n - 1;
    while (top >= 0 && mag[top] == 0) --top;
    if (top < 0) return 0;
    int L = 32 * (lo + top) + (31 - __builtin_clz(mag[top]));  // global bit of leading one
    int e_lead = L - kOffset;
    int lsb = std::max(e_lead - 112, -16494);
    int lp = lsb + kOffset;  // global bit position of the result lsb
    auto bit_at = [&](int g) -> uint32_t {
      int d = (g >> 5) - lo;
      if (g < 0 || d < 0 || d >= n) return 0;
      return (mag[d] >> (g & 31)) & 1;
    };
    u128 R = 0;
    for (int g = L; g >= lp; --g) R = (R << 1) | bit_at(g);
    uint32_t rbit = bit_at(lp - 1);
    bool st = false;
    int gb = lp - 2;  // highest sticky bit (global position)
    if (gb >= 32 * lo) {
      int d = (gb >> 5) - lo;
      uint32_t mask = (gb & 31) == 31 ? 0xffffffffu : ((1u << ((gb & 31) + 1)) - 1);
      if (d >= n) {  // a result far below the subnormal range: every digit is below gb
        d = n - 1;
        mask = 0xffffffffu;
      }
      st = (mag[d] & mask) != 0;
      for (int q = d - 1; q >= 0 && !st; --q) st = mag[q] != 0;
    }
    if (rbit && (st || (R & 1))) R += 1;
    if (R >> 113) {
      R >>= 1;
      lsb += 1;
    }
    oq v = (oq)(uint64_t)(R >> 64) * (oq)18446744073709551616.0 + (oq)(uint64_t)R;
    v = q_ldexp(v, lsb);
    return neg ? -v : v;
  }
};

// Exact sum_i x_i*y_i: R = round(S), r = round(S - R), absum = sum |x_i y_i|
// (computed in ordinary binary128 FMA arithmetic; used only for bounds).
static void exact_dot_core(LongAcc& acc, int64_t n, const oq* x, int64_t incx, const oq* y,
                           int64_t incy, oq* R, oq* r, oq* absum) {
  acc.clear();
  oq ab = 0;
  for (int64_t i = 0; i < n; ++i) {
    oq a = x[i * incx], b = y[i * incy];
    acc.add_product(a, b);
    ab = q_fma(q_fabs(a), q_fabs(b), ab);
  }
  oq Rv = acc.round();
  oq rv = 0;
  if (!q_isnan(Rv) && !q_isinf(Rv)) {
    acc.add_value(Rv, true);
    rv = acc.round();
  }
  if (R) *R = Rv;
  if (r) *r = rv;
  if (absum) *absum = ab;
}

void oq_exact_dot(int64_t n, const oq* x, int64_t incx, const oq* y, int64_t incy, oq* R, oq* r,
                  oq* absum) {
  LongAcc* acc = new LongAcc();
  exact_dot_core(*acc, n, x, incx, y, incy, R, r, absum);
  delete acc;
}

// Exact per-row sums of op(A) x, where op(A) is m x n: element (i, j) is
// A[i*si + j*sj].  (Row-major no-trans: si = lda, sj = 1.)
void oq_exact_gemv(int64_t m, int64_t n, const oq* A, int64_t si, int64_t sj, const oq* x,
                   int64_t incx, oq* R, oq* r, oq* absum, int nthreads) {
#pragma omp parallel num_threads(nthreads < 1 ? 1 : nthreads)
  {
    LongAcc* acc = new LongAcc();
#pragma omp for schedule(dynamic, 4)
    for (int64_t i = 0; i < m; ++i)
      exact_dot_core(*acc, n, &A[i * si], sj, x, incx, R ? &R[i] : nullptr, r ? &r[i] : nullptr,
                     absum ? &absum[i] : nullptr);
    delete acc;
  }
}

// Exact entries of op(A) op(B) for the listed (row, col) pairs.
// op(A)(i, l) = A[i*sai + l*sal]; op(B)(l, j) = B[l*sbl + j*sbj].
void oq_exact_gemm(int64_t k, const oq* A, int64_t sai, int64_t sal, const oq* B, int64_t sbl,
                   int64_t sbj, int64_t cnt, const int64_t* rows, const int64_t* cols, oq* R,
                   oq* r, oq* absum, int nthreads) {
#pragma omp parallel num_threads(nthreads < 1 ? 1 : nthreads)
  {
    LongAcc* acc = new LongAcc();
#pragma omp for schedule(dynamic, 16)
    for (int64_t t = 0; t < cnt; ++t) {
      int64_t i = rows[t], j = cols[t];
      exact_dot_core(*acc, k, &A[i * sai], sal, &B[j * sbj], sbl, R ? &R[t] : nullptr,
                     r ? &r[t] : nullptr, absum ? &absum[t] : nullptr);
    }
    delete acc;
  }
}

// Error of `got` against the exact value S = R + r, in units in the last
// place of R (binary128 ulp; 2^-16494 when R is zero or subnormal).
// Non-finite: 0 if got matches R's class (NaN) or value (inf), else +inf.
void oq_ulp_err(int64_t n, const oq* got, const oq* R, const oq* r, double* out) {
  for (int64_t i = 0; i < n; ++i) {
    oq g = got[i], Rv = R[i];
    if (q_isnan(Rv)) {
      out[i] = q_isnan(g) ? 0.0 : INFINITY;
      continue;
    }
    if (q_isinf(Rv)) {
      out[i] = (g == Rv) ? 0.0 : INFINITY;
      continue;
    }
    if (q_isnan(g) || q_isinf(g)) {
      out[i] = INFINITY;
      continue;
    }
    oq d = (g - Rv) - r[i];
    int ex = 0;
    if (Rv != 0) {
      uint64_t lo, hi;
      q_bits(Rv, lo, hi);
      int be = (int)((hi >> 48) & 0x7fff);
      ex = (be ? be - 16383 : -16382) - 112;
    } else {
      ex = -16494;
    }
    oq u = q_ldexp(q_fabs(d), -ex);
    double v = (double)u;
    out[i] = v;
  }
}

// ---------------------------------------------------------------------------
// 3. Ill-conditioned dot products of prescribed condition
// ---------------------------------------------------------------------------
// GenDot of Ogita, Rump and Oishi ("Accurate sum and dot product", SIAM J.
// Sci. Comput. 26(6), 2005, Algorithm 6.1), restated for binary128: the
// first half of x, y has random signs, random significands and exponents
// spread over [0, b/2] (b = log2(cond)), including both ends; in the second
// half the exponents fall linearly from b/2 to 0 and each y_i is chosen so
// that x_i*y_i nearly cancels the running exact sum, which the exact long
// accumulator provides (the paper uses a twice-working-precision dot).  The
// pairs are then permuted at random.  Deterministic for a given seed.
static inline uint64_t gd_next(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
// uniform in [-1, 1) with 106 random significand bits
static inline oq gd_unit(uint64_t& s) {
  const uint64_t hi = gd_next(s) >> 11;  // two statements: a fixed draw order
  const uint64_t lo = gd_next(s) >> 11;
  oq u = (oq)hi * q_ldexp((oq)1, -53) + (oq)lo * q_ldexp((oq)1, -106);
  return 2 * u - 1;
}

void oq_gendot(int64_t n, double cond, uint64_t seed, oq* x, oq* y) {
  uint64_t s = seed;
  LongAcc* acc = new LongAcc();
  const double b = log2(cond);
  const int64_t n2 = (n + 1) / 2;
  for (int64_t i = 0; i < n2; ++i) {
    int ex = (int)llround((double)(gd_next(s) >> 11) * 0x1p-53 * b / 2);
    int ey = (int)llround((double)(gd_next(s) >> 11) * 0x1p-53 * b / 2);
    if (i == 0) ex = ey = (int)llround(b / 2) + 1;
    if (i == n2 - 1) ex = ey = 0;
    x[i] = q_ldexp(gd_unit(s), ex);
    y[i] = q_ldexp(gd_unit(s), ey);
    acc->add_product(x[i], y[i]);
  }
  for (int64_t i = n2; i < n; ++i) {
    double frac = (n - 1 > n2) ? (double)(n - 1 - i) / (double)(n - 1 - n2) : 0.0;
    int e = (int)llround(b / 2 * frac);
    x[i] = q_ldexp(gd_unit(s), e);
    oq S = acc->round();
    y[i] = (q_ldexp(gd_unit(s), e) - S) / x[i];
    acc->add_product(x[i], y[i]);
  }
  for (int64_t i = n - 1; i > 0; --i) {
    int64_t j = (int64_t)(gd_next(s) % (uint64_t)(i + 1));
    oq t = x[i];
    x[i] = x[j];
    x[j] = t;
    t = y[i];
    y[i] = y[j];
    y[j] = t;
  }
  delete acc;
}

// `count` independent GenDot pairs: pair p (condition conds[p], seed
// seeds[p]) is written to X + p*n and Y + p*n.
void oq_gendot_batch(int64_t count, int64_t n, const double* conds, const uint64_t* seeds, oq* X,
                     oq* Y, int nthreads) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
  for (int64_t p = 0; p < count; ++p) oq_gendot(n, conds[p], seeds[p], X + p * n, Y + p * n);
}

// Condition number 2 * sum|x_i y_i| / |sum x_i y_i| of a dot product (double).
double oq_dot_condition(int64_t n, const oq* x, int64_t incx, const oq* y, int64_t incy) {
  oq R, r, ab;
  oq_exact_dot(n, x, incx, y, incy, &R, &r, &ab);
  return (double)(2 * ab / q_fabs(R));
}

// Counts entries with |got - ref| > kfac * 2^-113 * absum (the reduction
// bound k * u_q * sum|a_i b_i| with u_q = 2^-113); NaN/inf must match.
int64_t oq_count_bound_violations(int64_t n, const oq* got, const oq* ref, const oq* absum,
                                  double kfac) {
  int64_t bad = 0;
  for (int64_t i = 0; i < n; ++i) {
    oq g = got[i], f = ref[i];
    if (q_isnan(f) || q_isnan(g)) {
      bad += !(q_isnan(f) && q_isnan(g));
      continue;
    }
    if (q_isinf(f) || q_isinf(g)) {
      bad += !(g == f);
      continue;
    }
    oq lim = q_ldexp((oq)kfac * absum[i], -113);
    if (q_fabs(g - f) > lim) ++bad;
  }
  return bad;
}

}  // extern "C"
