// Test harness: the device soft-float core (qblas_gb300/csrc/softquad.cuh)
// compiled as plain host C++, so its bit patterns can be compared with the
// host binary128 library on a machine without a GPU.
#include <string.h>
#include <stdint.h>

#include "../qblas_gb300/csrc/softquad.cuh"
#include "../qblas_gb300/csrc/wacc.cuh"
#include "../qblas_gb300/csrc/ozaki.cuh"
#include "../qblas_gb300/csrc/exact.cuh"
#include "../qblas_gb300/csrc/ozgemv.cuh"
#include "../qblas_gb300/csrc/ozcrt.cuh"

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
void sq_epilogue_n(int64_t n, const q128* alpha, const q128* sum, const q128* beta, const q128* y, q128* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = qb::q_epilogue(alpha[i], sum[i], beta[i], y[i]);
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
// As sq_wacc_dot_certified with the truncated products of the qdot kernel
// (mul128x128_top192) and its budget of 2^34 + 2 units per product.
void sq_wacc_dot_trunc_certified(int64_t n, const q128* x, const q128* y, int64_t nsplit, q128* out,
                                 int32_t* certified) {
  qb::wacc tot;
  qb::wacc_init(tot);
  if (nsplit < 1) nsplit = 1;
  int64_t chunk = (n + nsplit - 1) / nsplit;
  for (int64_t s = 0; s < nsplit; ++s) {
    qb::wacc a;
    qb::wacc_init(a);
    for (int64_t i = s * chunk; i < n && i < (s + 1) * chunk; ++i)
      qb::wacc_add_product_trunc(a, qb::qop_unpack(x[i]), qb::qop_unpack(y[i]));
    qb::wacc_merge(tot, a);
  }
  const uint64_t err = (uint64_t)n * ((1ull << 34) + 2) + 3 * (uint64_t)nsplit + 3;
  *certified = qb::wacc_round_certified(tot, err, *out) ? 1 : 0;
}
// Limbs 2..7 of the truncated significand product (mul128x128_top192) of
// n pairs, six words each.
void sq_mul_top192(int64_t n, const q128* x, const q128* y, uint32_t* out) {
  for (int64_t i = 0; i < n; ++i) {
    qb::qop a = qb::qop_unpack(x[i]), b = qb::qop_unpack(y[i]);
    qb::mul128x128_top192(a, b, out[6 * i], out[6 * i + 1], out[6 * i + 2], out[6 * i + 3], out[6 * i + 4],
                          out[6 * i + 5]);
  }
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
// Ozaki qgemv arithmetic (ozgemv.cuh): windows W of n elements against
// exponents E[i] (five words each).
void sq_og_window(int64_t n, const q128* a, const int32_t* E, uint32_t* W) {
  for (int64_t i = 0; i < n; ++i) {
    uint32_t w[5];
    qb::og_window((uint32_t)a[i].lo, (uint32_t)(a[i].lo >> 32), (uint32_t)a[i].hi,
                  (uint32_t)(a[i].hi >> 32), E[i], w);
    for (int k = 0; k < 5; ++k) W[5 * i + k] = w[k];
  }
}
static int og_lead_x(const q128& x) {  // nonzero finite x: its lead exponent; else kOgNoExp
  const uint32_t top = (uint32_t)(x.hi >> 32);
  if (qb::og_special_top(top)) return qb::kOgNoExp;
  if (((x.hi & 0x7FFFFFFFFFFFFFFFull) | x.lo) == 0) return qb::kOgNoExp;
  return qb::og_lead_top(top);
}
// One chunk (n <= 32 terms): E, F, the diagonal sums D[0..31] and T.
void sq_og_chunk(int n, const q128* a, const q128* x, int32_t* EF, int64_t* D, uint32_t* T) {
  int E = -16382, F = qb::kOgNoExp;
  for (int j = 0; j < n; ++j) {
    int l = qb::og_lead_top((uint32_t)(a[j].hi >> 32));
    E = l > E ? l : E;
    int f = og_lead_x(x[j]);
    F = f > F ? f : F;
  }
  for (int g = 0; g < 32; ++g) D[g] = 0;
  for (int j = 0; j < n; ++j) {
    uint32_t wa[5], wx[5];
    qb::og_window((uint32_t)a[j].lo, (uint32_t)(a[j].lo >> 32), (uint32_t)a[j].hi, (uint32_t)(a[j].hi >> 32), E, wa);
    qb::og_window((uint32_t)x[j].lo, (uint32_t)(x[j].lo >> 32), (uint32_t)x[j].hi, (uint32_t)(x[j].hi >> 32),
                  F == qb::kOgNoExp ? -16382 : F, wx);
    for (int t = 0; t < qb::kOgPlanes; ++t)
      for (int u = 0; u < qb::kOgPlanes; ++u)
        if (t + u < 32)
          D[t + u] += (int64_t)qb::og_digit(wa, t, (uint32_t)(a[j].hi >> 63)) *
                      qb::og_digit(wx, u, (uint32_t)(x[j].hi >> 63));
  }
  int32_t D32[qb::kOgDiags];
  for (int g = 0; g < qb::kOgDiags; ++g) D32[g] = (int32_t)D[g];
  uint32_t t6[6];
  qb::og_fold(D32, t6);
  for (int k = 0; k < 6; ++k) T[k] = t6[k];
  EF[0] = E;
  EF[1] = F;
}
// Windows by the short form (valid for shifts below 128), else 0xFFFFFFFF.
void sq_og_window_short(int64_t n, const q128* a, const int32_t* E, uint32_t* W) {
  for (int64_t i = 0; i < n; ++i) {
    const uint32_t w3 = (uint32_t)(a[i].hi >> 32);
    const int s = qb::og_shift(E[i], w3);
    uint32_t w[5] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
    if (s < 128) qb::og_window_s<true>((uint32_t)a[i].lo, (uint32_t)(a[i].lo >> 32), (uint32_t)a[i].hi, w3, s, w);
    for (int k = 0; k < 5; ++k) W[5 * i + k] = w[k];
  }
}
// The work partition of the Ozaki qgemv kernel: begin[b] for b = 0..G and
// cta[X] for every item X < work.
void sq_og_partition(int64_t work, int64_t G, int64_t* begin, int64_t* cta) {
  for (int64_t b = 0; b <= G; ++b) begin[b] = qb::og_range_begin(work, G, b);
  for (int64_t X = 0; X < work; ++X) cta[X] = qb::og_cta_of(work, G, X);
}
// A whole row the way the kernels treat it (one partial, no merges):
// out = the certified rounding, returns 1 when certified, 0 otherwise.
int sq_og_row(int64_t n, const q128* a, const q128* x, q128* out) {
  qb::wacc acc;
  qb::wacc_init(acc);
  const int kNone = 2 * qb::kOgNoExp;
  int gmax = kNone;
  uint32_t nch = 0;
  bool spec = false;
  for (int64_t j0 = 0; j0 < n; j0 += qb::kOgChunk) {
    const int c = (int)(n - j0 < qb::kOgChunk ? n - j0 : qb::kOgChunk);
    for (int j = 0; j < c; ++j) spec = spec || qb::og_special_top((uint32_t)(a[j0 + j].hi >> 32)) ||
                                         qb::og_special_top((uint32_t)(x[j0 + j].hi >> 32));
    int32_t EF[2];
    int64_t D[32];
    uint32_t T[6];
    sq_og_chunk(c, a + j0, x + j0, EF, D, T);
    ++nch;
    if (EF[1] == qb::kOgNoExp) continue;
    gmax = EF[0] + EF[1] > gmax ? EF[0] + EF[1] : gmax;
    qb::og_wacc_add(acc, T, EF[0] + EF[1] - qb::kOgFoldShift);
  }
  if (spec) return 0;
  if (gmax == kNone) {
    *out = qb::wacc_round(acc);  // every product is an exact zero
    return 1;
  }
  if (acc.e == qb::kWaccEmptyExp) return 0;
  uint64_t err = qb::og_row_error(acc, nch, gmax, 0);
  return qb::wacc_round_certified(acc, err, *out) ? 1 : 0;
}

// ---- Ozaki scheme II (ozcrt.cuh) ------------------------------------------
// The table for T-bit operands and inner dimension k: returns n (moduli) or 0,
// and writes n, nw, then p, u, c18[11] per modulus, then Mpair[24][12] and
// negM[12] as uint32 (out must hold 4 + 48 * 13 + 24 * 12 + 12 words).
int sq_crt_table(int T, int64_t k, uint32_t* out) {
  qb::CrtTable t;
  if (!qb::crt_build(T, k, t)) return 0;
  int o = 0;
  out[o++] = (uint32_t)t.n;
  out[o++] = (uint32_t)t.nw;
  out[o++] = (uint32_t)t.T;
  out[o++] = 0;
  for (int q = 0; q < qb::kCrtMaxMods; ++q) {
    out[o++] = t.mod[q].p;
    out[o++] = t.mod[q].u;
    for (int j = 0; j < qb::kCrtPieces; ++j) out[o++] = t.mod[q].c18[j];
  }
  for (int i = 0; i < qb::kCrtMaxMods / 2; ++i)
    for (int w = 0; w < qb::kCrtMaxWords; ++w) out[o++] = t.Mpair[i][w];
  for (int w = 0; w < qb::kCrtMaxWords; ++w) out[o++] = t.negM[w];
  return t.n;
}

// x mod p by the magic multiplier, for x[i], i < n.
void sq_crt_mod(int64_t n, const uint32_t* x, uint32_t p, uint32_t* r) {
  const uint32_t magic = (uint32_t)(((1ull << 40) + p - 1) / p);
  for (int64_t i = 0; i < n; ++i) r[i] = qb::crt_mod(x[i], p, magic);
}

// Balanced residues r[i][q] (sign included) of a[i] for scale S and T bits,
// and the scaled integer V (3 words) with its sign.
int sq_crt_residues(int64_t n, const q128* a, const int* S, int T, int64_t k, int* r, uint64_t* V) {
  qb::CrtTable t;
  if (!qb::crt_build(T, k, t)) return 0;
  for (int64_t i = 0; i < n; ++i) {
    qb::crt_residues(a[i], S[i], t, r + i * t.n);
    bool neg;
    qb::ozaki_scaled_bits(a[i], S[i], T, V[4 * i], V[4 * i + 1], V[4 * i + 2], neg);
    V[4 * i + 3] = neg;
  }
  return t.n;
}

// The tensor-core residue split's table for T-bit operands and inner
// dimension k: header {nmod, N, NB, T}, p and 1/p as fp32 bit patterns
// (kCrtMaxMods each), and the B operand (kCrtSplitK x kCrtSplitMaxN fp16
// bit patterns in the shared-memory layout).  Returns the number of moduli.
int sq_crt_split_table(int T, int64_t k, int32_t* head4, uint32_t* p_bits, uint32_t* inv_bits, uint16_t* b) {
  qb::CrtTable t;
  if (!qb::crt_build(T, k, t)) return 0;
  qb::CrtSplitTable st;
  qb::crt_split_table(t, st);
  head4[0] = st.nmod;
  head4[1] = st.N;
  head4[2] = st.NB;
  head4[3] = st.T;
  memcpy(p_bits, st.p, sizeof(st.p));
  memcpy(inv_bits, st.inv_p, sizeof(st.inv_p));
  memcpy(b, st.b, sizeof(st.b));
  return t.n;
}

// crt_scaled_words (6 words) and ozaki_scaled_bits of each a[i] with scale
// S[i]: out[i] = {6 words, neg} and ref[i] = {v0, v1, v2, neg}.
void sq_crt_scaled_words(int64_t n, const q128* a, const int* S, int T, uint32_t* out, uint64_t* ref) {
  for (int64_t i = 0; i < n; ++i) {
    uint32_t w[6];
    bool neg;
    qb::crt_scaled_words<6>(a[i], S[i], T, w, neg);
    for (int j = 0; j < 6; ++j) out[7 * i + j] = w[j];
    out[7 * i + 6] = neg;
    bool neg2;
    qb::ozaki_scaled_bits(a[i], S[i], T, ref[4 * i], ref[4 * i + 1], ref[4 * i + 2], neg2);
    ref[4 * i + 3] = neg2;
  }
}

// The tensor-core reconstruction for outputs whose residue sums are C[i][q]
// (one pass): y_q reduced as the product kernel stores it, the column sums
// Z_w = sum_q y_q B[w][q] taken from the fp16 table (decoded here, exact
// integers), then crt_fold_columns; also returns the largest Z seen.
static int half_int(uint16_t h) {
  if ((h & 0x7FFF) == 0) return 0;
  const int e = (h >> 10) & 0x1F, m = (h & 0x3FF) | 0x400;
  const int v = e >= 25 ? m << (e - 25) : m >> (25 - e);
  return (h & 0x8000) ? -v : v;
}
extern "C++" {
template <int NW>
static q128 fold_biased(const uint32_t* Z, const qb::CrtFoldTable& ft, int e) {
  qb::CrtFoldAcc<NW> A;
  qb::crt_fold_init(A);
  for (int w = 0; w < ft.N; ++w) {
    float f = (float)Z[w] + 8388608.0f;
    uint32_t bits;
    memcpy(&bits, &f, 4);
    qb::crt_fold_column(A, w, bits, true);
  }
  return qb::crt_fold_finish(A, ft.negM, e, true);
}
}

int sq_crt_fold_tc(int64_t n, const int32_t* C, const int* e, int T, int64_t k, q128* out, int64_t* zmax) {
  qb::CrtTable t;
  if (!qb::crt_build(T, k, t)) return 0;
  qb::CrtFoldTable ft;
  qb::crt_fold_table(t, ft);
  *zmax = 0;
  for (int64_t i = 0; i < n; ++i) {
    uint32_t y[qb::kCrtMaxMods] = {0};
    for (int q = 0; q < t.n; ++q) y[q] = qb::crt_y(qb::crt_reduce(C[i * t.n + q], t.mod[q]), t.mod[q]);
    uint32_t Z[qb::kCrtFoldMaxN] = {0};
    for (int col = 0; col < ft.N; ++col) {
      int64_t z = 0;
      for (int q = 0; q < qb::kCrtFoldK; ++q)
        z += (int64_t)y[q] * half_int(ft.b[(q / 8) * (ft.N * 8) + col * 8 + (q % 8)]);
      if (z > *zmax) *zmax = z;
      Z[col] = (uint32_t)z;
    }
    q128 r;
    if (ft.nw <= 8)
      r = qb::crt_fold_columns<8>(Z, ft.nbytes, ft.negM, e[i]);
    else if (ft.nw <= 10)
      r = qb::crt_fold_columns<10>(Z, ft.nbytes, ft.negM, e[i]);
    else
      r = qb::crt_fold_columns<12>(Z, ft.nbytes, ft.negM, e[i]);
    // the kernel's form: each sum as the bits of the fp32 value 2^23 + z, the
    // offsets taken off per word
    q128 rb;
    if (ft.nw <= 8)
      rb = fold_biased<8>(Z, ft, e[i]);
    else if (ft.nw <= 10)
      rb = fold_biased<10>(Z, ft, e[i]);
    else
      rb = fold_biased<12>(Z, ft, e[i]);
    if (rb.lo != r.lo || rb.hi != r.hi) return -1;
    out[i] = r;
  }
  return t.n;
}

// Reconstruction of X 2^e[i] from C[i][q] (one pass) for each output i.
int sq_crt_reconstruct(int64_t n, const int32_t* C, const int* e, int T, int64_t k, q128* out) {
  qb::CrtTable t;
  if (!qb::crt_build(T, k, t)) return 0;
  for (int64_t i = 0; i < n; ++i) out[i] = qb::crt_reconstruct_any(C + i * t.n, t, e[i]);
  return t.n;
}

// CRT split of a view as the device does it: row scales S[r] and balanced
// residues R[q][r][c] for T-bit operands and the table of inner dimension k.
int sq_crt_split(int64_t rows, int64_t cols, const q128* X, int64_t sr, int64_t sc, int T, int64_t k,
                 int32_t* S, int32_t* R) {
  qb::CrtTable t;
  if (!qb::crt_build(T, k, t)) return 0;
  int r_q[qb::kCrtMaxMods];
  for (int64_t r = 0; r < rows; ++r) {
    int mx = qb::kOzakiScaleEmpty;
    for (int64_t c = 0; c < cols; ++c) {
      int e = qb::ozaki_exp_plus1(X[r * sr + c * sc]);
      mx = e > mx ? e : mx;
    }
    S[r] = mx;
    for (int64_t c = 0; c < cols; ++c) {
      qb::crt_residues(X[r * sr + c * sc], mx, t, r_q);
      for (int q = 0; q < t.n; ++q) R[((int64_t)q * rows + r) * cols + c] = r_q[q];
    }
  }
  return t.n;
}

// CRT reconstruction of exact residue-product sums C[q][i][j] (int64) with
// scales S[i], F[j].
int sq_crt_fold(int64_t m, int64_t n, int T, int64_t k, const int64_t* C, const int32_t* S, const int32_t* F,
                q128* out) {
  qb::CrtTable t;
  if (!qb::crt_build(T, k, t)) return 0;
  int32_t c[qb::kCrtMaxMods];
  for (int64_t i = 0; i < m; ++i)
    for (int64_t j = 0; j < n; ++j) {
      for (int q = 0; q < t.n; ++q) {
        const int64_t p = t.mod[q].p, v = C[((int64_t)q * m + i) * n + j] % p;
        c[q] = (int32_t)(v < 0 ? v + p : v);
      }
      out[i * n + j] = qb::crt_reconstruct_any(c, t, S[i] + F[j] - 2 * T);
    }
  return t.n;
}
}  // extern "C"
