// Test harness: the device soft-float core (qblas_gb300/csrc/softquad.cuh)
// compiled as plain host C++, so its bit patterns can be compared with the
// host binary128 library on a machine without a GPU.
#include <stdint.h>

#include "../qblas_gb300/csrc/softquad.cuh"
#include "../qblas_gb300/csrc/wacc.cuh"
#include "../qblas_gb300/csrc/ozaki.cuh"
#include "../qblas_gb300/csrc/exact.cuh"

using qb::q128;

extern "C" {
void sq_fma_n(int64_t n, const q128* a, const q128* b, const q128* c, q128* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = qb::q_fma(a[i], b[i], c[i]);
}
void sq_mul_n(int64_t n, const q128* a, const q128* b, q128* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = qb::q_mul(a[i], b[i]);
}
void sq_add_n(int64_t n, const q128* a, const q128* b, q128* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = qb::q_add(a[i], b[i]);
}
void sq_sub_n(int64_t n, const q128* a, const q128* b, q128* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = qb::q_sub(a[i], b[i]);
}
void sq_sqrt_n(int64_t n, const q128* a, q128* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = qb::q_sqrt(a[i]);
}
void sq_from_double_n(int64_t n, const uint64_t* d, q128* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = qb::q_from_double_bits(d[i]);
}
void sq_to_double_n(int64_t n, const q128* a, uint64_t* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = qb::q_to_double_bits(a[i]);
}
// Dot product through the wide accumulator: the n terms are cut into
// `nsplit` contiguous chunks, each accumulated separately, then merged in
// order (the structure of the device reduction).
void sq_wacc_dot(int64_t n, const q128* x, int64_t incx, const q128* y, int64_t incy, int64_t nsplit,
                 q128* out) {
  qb::wacc tot;
  qb::wacc_init(tot);
  if (nsplit < 1) nsplit = 1;
  int64_t chunk = (n + nsplit - 1) / nsplit;
  for (int64_t s = 0; s < nsplit; ++s) {
    qb::wacc a;
    qb::wacc_init(a);
    for (int64_t i = s * chunk; i < n && i < (s + 1) * chunk; ++i)
      qb::wacc_add_product(a, qb::qop_unpack(x[i * incx]), qb::qop_unpack(y[i * incy]));
    qb::wacc_merge(tot, a);
  }
  *out = qb::wacc_round(tot);
}
// The wide-accumulator dot as above plus its rounding certificate for the
// error budget of n products and nsplit merges (2n + 3 nsplit units).
void sq_wacc_dot_certified(int64_t n, const q128* x, const q128* y, int64_t nsplit, q128* out,
                           int32_t* certified) {
  qb::wacc tot;
  qb::wacc_init(tot);
  if (nsplit < 1) nsplit = 1;
  int64_t chunk = (n + nsplit - 1) / nsplit;
  for (int64_t s = 0; s < nsplit; ++s) {
    qb::wacc a;
    qb::wacc_init(a);
    for (int64_t i = s * chunk; i < n && i < (s + 1) * chunk; ++i)
      qb::wacc_add_product(a, qb::qop_unpack(x[i]), qb::qop_unpack(y[i]));
    qb::wacc_merge(tot, a);
  }
  *certified = qb::wacc_round_certified(tot, 2 * (uint64_t)n + 3 * (uint64_t)nsplit + 3, *out) ? 1 : 0;
}
// Exact dot through the Kulisch accumulator (the device fallback's arithmetic).
void sq_kulisch_dot(int64_t n, const q128* x, int64_t incx, const q128* y, int64_t incy, q128* out) {
  static int64_t d[qb::kKDigits];
  for (int i = 0; i < qb::kKDigits; ++i) d[i] = 0;
  int lo = qb::kKDigits, hi = -1;
  uint32_t flags = 0;
  for (int64_t i = 0; i < n; ++i) {
    qb::qop a = qb::qop_unpack(x[i * incx]), b = qb::qop_unpack(y[i * incy]);
    if ((a.cls | b.cls) != qb::kClsFinite)
      flags |= qb::special_product_flags(a, b);
    else
      qb::kulisch_add_product(d, a, b, lo, hi);
  }
  if (lo > hi) lo = hi = 0;
  int64_t carry = qb::kulisch_normalize(d, lo, hi);
  *out = qb::kulisch_round(d, lo, hi, carry, flags);
}
// Ozaki split of a rows x cols view X(r, c) = X[r*sr + c*sc]: row scales
// S[r] and digits D[t][r][c] (int32), the device kernels' arithmetic.
void sq_ozaki_split(int64_t rows, int64_t cols, const q128* X, int64_t sr, int64_t sc, int s,
                    int b, int32_t* S, int32_t* D) {
  for (int64_t r = 0; r < rows; ++r) {
    int mx = qb::kOzakiScaleEmpty;
    for (int64_t c = 0; c < cols; ++c) {
      int e = qb::ozaki_exp_plus1(X[r * sr + c * sc]);
      mx = e > mx ? e : mx;
    }
    S[r] = mx;
    for (int64_t c = 0; c < cols; ++c) {
      int dg[qb::kOzakiMaxDigits];
      qb::ozaki_digits(X[r * sr + c * sc], mx, s, b, dg);
      for (int t = 0; t < s; ++t) D[((int64_t)t * rows + r) * cols + c] = dg[t];
    }
  }
}
// Fold of diagonals C[g][i][j] (int64, g <= G) with scales S[i], F[j].
void sq_ozaki_fold(int64_t m, int64_t n, int G, int b, const int64_t* C, const int32_t* S,
                   const int32_t* F, q128* out) {
  for (int64_t i = 0; i < m; ++i)
    for (int64_t j = 0; j < n; ++j) {
      qb::fold192 f;
      qb::fold_init(f);
      for (int g = 0; g <= G; ++g) qb::fold_step(f, C[((int64_t)g * m + i) * n + j], b);
      out[i * n + j] = qb::fold_round(f, qb::ozaki_fold_exp(S[i], F[j], G, b));
    }
}
}
