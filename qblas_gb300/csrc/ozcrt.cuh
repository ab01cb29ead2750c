// Ozaki scheme II for qgemm: exact integer products through residues.
//
// Published method: K. Ozaki, Y. Uchino, T. Imamura, "Ozaki Scheme II: A
// GEMM-oriented emulation of floating-point matrix multiplication using an
// integer modular technique" (2025).  Restated here for binary128 operands
// and fp16 digit products on the tensor cores.
//
// Rows of op(A) are scaled as in the digit split (ozaki.cuh): with S_i the
// row scale, a_il becomes the integer A'_il = sign * trunc(|a_il| 2^(T-S_i)),
// |A'| < 2^T, and the columns of op(B) likewise (scale F_j).  The exact
// integer X_ij = sum_l A'_il B'_lj (|X| < k 2^(2T)) is then computed modulo N
// pairwise coprime moduli p_q in (256, 513]: for each q the balanced
// residues of A' and B' (|r| <= 256, exact in fp16) are multiplied on the
// tensor cores (an fp32 sum of 256 products of at most 2^16 is exact), and
// C_q = sum_l r_q(A'_il) r_q(B'_lj) == X_ij (mod p_q).  With M = prod p_q >
// (65/32) k 2^(2T), the Chinese remainder theorem gives X_ij back exactly:
//     Y = sum_q y_q M / p_q,   y_q = (C_q mod p_q) (M / p_q)^-1 mod p_q,
//     X = Y - Q M,             Q = round(sum_q y_q / p_q),
// and sum_l a_il b_lj ~= X 2^(S_i + F_j - 2T) is rounded once.  The only
// error is the truncation of the operands to T bits, the same truncation as
// the digit split with b*s - 1 = T bits, without its dropped digit pairs; the
// number of tensor-core products is N (about (2T + log2 k + 1) / 8.9) instead
// of s(s+1)/2.
#pragma once
#include <stdint.h>
#include <string.h>

#include "ozaki.cuh"
#include "wacc.cuh"

namespace qb {

constexpr int kCrtMaxMods = 48;    // moduli (about 414 bits)
constexpr int kCrtMaxWords = 12;   // 32-bit words of the reconstruction (384 bits)
constexpr int kCrtPieces = 11;     // 18-bit pieces of a scaled operand (T <= 191)
constexpr int kCrtPassK = 8192;    // k per pass: |C_q| <= 8192 * 2^16 = 2^29

struct alignas(16) CrtMod {
  uint32_t p;      // modulus, 257..513
  uint32_t magic;  // ceil(2^40 / p): x mod p = x - p ((x magic) >> 40) for x < 2^40 / 513
  uint32_t K;      // p ceil(2^29 / p): c + K >= 0 for |c| <= 2^29
  uint32_t u;      // (M / p)^-1 mod p
  uint32_t P24;    // round(2^24 / p), for the estimate of Q
  uint32_t half;   // floor(p / 2): balanced residues are ((x + half) mod p) - half
  uint32_t bias2;  // (0x6600 - half) * 0x10001: two shifted residues to fp16 bits 0x6600 + r
  uint32_t pad;
  uint32_t c18[kCrtPieces];  // 2^(18 j) mod p
  uint32_t pad2;
};

// 16-byte aligned (also as a kernel parameter): the kernels copy it with
// 16-byte loads.
struct alignas(16) CrtTable {
  int n;   // moduli in use
  int nw;  // 32-bit words of the reconstruction (8, 10 or 12; M < 2^(32 nw))
  int T;   // |A'|, |B'| < 2^T
  int pad;
  CrtMod mod[kCrtMaxMods];
  // M / (p_2i p_2i+1) (M / p_2i for a last unpaired modulus), little-endian words
  uint32_t Mpair[kCrtMaxMods / 2][kCrtMaxWords];
  uint32_t negM[kCrtMaxWords];  // 2^(32 nw) - M
};
static_assert(sizeof(CrtMod) == 80 && sizeof(CrtTable) <= 8192, "CRT table layout (a kernel parameter)");

// ---------------------------------------------------------------------------
// Host: the moduli and the table
// ---------------------------------------------------------------------------
// Pairwise coprime moduli, greedily from 513 down: 513, 512, 511, 509, 505,
// 503, 499, 493, ... (50 of them above 256).
inline int crt_moduli(uint32_t* out, int cap) {
  int n = 0;
  for (uint32_t p = 513; p > 256 && n < cap; --p) {
    bool ok = true;
    for (int i = 0; i < n && ok; ++i) {
      uint32_t a = p, b = out[i];
      while (b) {
        const uint32_t t = a % b;
        a = b;
        b = t;
      }
      ok = a == 1;
    }
    if (ok) out[n++] = p;
  }
  return n;
}

// little-endian multiword helpers (host)
inline void crt_big_mul_small(uint32_t* w, int nw, uint32_t f) {
  uint64_t c = 0;
  for (int i = 0; i < nw; ++i) {
    c += (uint64_t)w[i] * f;
    w[i] = (uint32_t)c;
    c >>= 32;
  }
}

inline int crt_big_bits(const uint32_t* w, int nw) {
  for (int i = nw - 1; i >= 0; --i)
    if (w[i]) {
      int b = 32;
      while (!((w[i] >> (b - 1)) & 1u)) --b;
      return 32 * i + b;
    }
  return 0;
}

inline uint32_t crt_inverse(uint32_t a, uint32_t p) {  // a^-1 mod p, gcd(a, p) = 1
  int64_t t = 0, nt = 1, r = p, nr = a % p;
  while (nr) {
    const int64_t q = r / nr, tt = t - q * nt, rr = r - q * nr;
    t = nt;
    nt = tt;
    r = nr;
    nr = rr;
  }
  return (uint32_t)(t < 0 ? t + p : t);
}

// The moduli product M must exceed (65/32) k 2^(2T) for operands of T bits
// and inner dimension k.  Then |X| < k 2^(2T) < (32/65) M, and Q is the
// integer nearest to Y / M = Q + X / M.  Its estimate S 2^-24, S = sum_q y_q
// P24_q with |P24_q - 2^24 / p_q| <= 1/2 and y_q <= 512, is off by at most
// n 2^-16 <= 48 2^-16 < 7.4e-4 from Y / M; |X / M| + 7.4e-4 < 32/65 + 7.4e-4
// < 1/2, so rounding S 2^-24 gives Q.
//
// True when 32 M > 65 k 2^(2T) (M over `mw` little-endian words, k < 2^48,
// 65 k 2^(2T) below 2^(32 mw)).
inline bool crt_product_enough(const uint32_t* M, int mw, int T, int64_t k) {
  uint32_t lhs[kCrtMaxWords + 3] = {0}, rhs[kCrtMaxWords + 3] = {0};
  for (int w = 0; w < mw && w < kCrtMaxWords + 2; ++w) lhs[w] = M[w];
  crt_big_mul_small(lhs, kCrtMaxWords + 3, 32u);
  const uint64_t f = 65ull * (uint64_t)k;  // < 2^55
  const int sh = 2 * T;
  const int w0 = sh / 32, b0 = sh % 32;
  const uint32_t parts[2] = {(uint32_t)f, (uint32_t)(f >> 32)};
  for (int i = 0; i < 2; ++i) {
    const uint64_t v = (uint64_t)parts[i] << b0;
    if (w0 + i < kCrtMaxWords + 3) rhs[w0 + i] |= (uint32_t)v;
    if (w0 + i + 1 < kCrtMaxWords + 3) rhs[w0 + i + 1] |= (uint32_t)(v >> 32);
  }
  for (int w = kCrtMaxWords + 2; w >= 0; --w)
    if (lhs[w] != rhs[w]) return lhs[w] > rhs[w];
  return false;
}

// Fills `tab` for T-bit operands and inner dimension k; false when more than
// kCrtMaxMods moduli or kCrtMaxWords words would be needed (or T > 191, or
// k >= 2^48).
inline bool crt_build(int T, int64_t k, CrtTable& tab) {
  if (T < 2 || T > 191 || k < 1 || k >= ((int64_t)1 << 48)) return false;
  uint32_t P[64];
  const int avail = crt_moduli(P, 64);
  uint32_t M[kCrtMaxWords + 2] = {1};
  int n = 0;
  while (!crt_product_enough(M, kCrtMaxWords + 2, T, k)) {
    if (n == kCrtMaxMods || n == avail) return false;
    crt_big_mul_small(M, kCrtMaxWords + 2, P[n++]);
  }
  int nw = (crt_big_bits(M, kCrtMaxWords + 2) + 31) / 32;
  nw += nw & 1;
  if (nw < 8) nw = 8;  // the reconstruction runs on 8, 10 or 12 words
  if (nw > kCrtMaxWords) return false;
  tab = CrtTable();
  tab.n = n;
  tab.nw = nw;
  tab.T = T;
  for (int q = 0; q < n; ++q) {
    CrtMod& m = tab.mod[q];
    const uint32_t p = P[q];
    m.p = p;
    m.magic = (uint32_t)(((1ull << 40) + p - 1) / p);
    m.K = p * (uint32_t)(((1u << 29) + p - 1) / p);
    m.P24 = (uint32_t)(((1u << 24) + p / 2) / p);
    m.half = p / 2;
    m.bias2 = (0x6600u - p / 2) * 0x10001u;
    uint32_t c = 1 % p;
    for (int j = 0; j < kCrtPieces; ++j) {
      m.c18[j] = c;
      c = (uint32_t)(((uint64_t)c << 18) % p);
    }
    uint64_t Mq = 1;  // (M / p) mod p
    for (int r = 0; r < n; ++r)
      if (r != q) Mq = Mq * P[r] % p;
    m.u = crt_inverse((uint32_t)Mq, p);
  }
  for (int i = 0; 2 * i < n; ++i) {
    uint32_t W[kCrtMaxWords + 2] = {1};
    for (int r = 0; r < n; ++r)
      if (r != 2 * i && r != 2 * i + 1) crt_big_mul_small(W, kCrtMaxWords + 2, P[r]);
    for (int w = 0; w < kCrtMaxWords; ++w) tab.Mpair[i][w] = w < nw ? W[w] : 0u;
  }
  uint64_t b = 1;  // 2^(32 nw) - M = ~M + 1 over nw words
  for (int w = 0; w < nw; ++w) {
    b += (uint64_t)(uint32_t)~M[w];
    tab.negM[w] = (uint32_t)b;
    b >>= 32;
  }
  return true;
}

// ---------------------------------------------------------------------------
// Residue split on the tensor cores: the table (host)
// ---------------------------------------------------------------------------
// For the split kernel, an element's scaled integer V (NB bytes b_j, V =
// sum_j b_j 256^j, NB = 18 for T <= 144 and 24 for T <= 191) becomes 32
// values of one row of an MMA operand A: the fp16 values s (1024 + b_j) (one
// byte select each: the bits 0x64 | sign above the byte), then -s, then
// zeros (s = +-1 the sign of the element).  B holds, per modulus q, the
// balanced c_jq = 256^j mod p_q and beta_q = (1024 sum_j c_jq) mod p_q, both
// of magnitude at most 256, so that
//   x_q = s sum_j (1024 + b_j) c_jq - s beta_q == s V  (mod p_q),
//   |x_q| <= NB * 1279 * 256 + 256 < 2^23,
// an integer the fp32 accumulation holds exactly.  The balanced residue is
// then r = x - p * round(x / p) in fp32: the error of x * fl(1/p) is below
// |x| 2^-33 < 9.2e-4, less than the distance 1 / (2p) >= 9.78e-4 of x / p
// from a half-integer for odd p, so round() picks the nearest integer and
// |r| <= floor(p / 2) (for p = 512 a tie gives +-256).  Two elements share
// an operand row (K = 32 each) with block-diagonal B (N = 2 NP columns,
// element e of modulus q in column 2q + e, NP = nmod rounded up to 8).
constexpr int kCrtSplitK = 64;                   // K: 32 per element, two elements
constexpr int kCrtSplitMaxN = 2 * kCrtMaxMods;   // 96

struct alignas(16) CrtSplitTable {
  int nmod, N, NB, T;
  float p[kCrtMaxMods];
  float inv_p[kCrtMaxMods];
  // the same as pairs for the packed fp32 arithmetic (two elements at once):
  // (fl(1/p), fl(1/p)) and (-p, -p) as the bits of two floats, low one first
  uint64_t inv_p2[kCrtMaxMods];
  uint64_t neg_p2[kCrtMaxMods];
  // B in the shared-memory layout of a K-major operand without swizzle: the
  // 16 bytes of (row n, k-block kb) at kb * (N * 16) + n * 16
  uint16_t b[kCrtSplitK * kCrtSplitMaxN];
};

// The 32-bit words of V = trunc(|a| 2^(T - S)) (as ozaki_scaled_bits) for
// the split kernel, without data-dependent branches on the common path:
// |a| = M 2^(E - 112) with M the 113-bit significand (subnormals are
// normalised in a branch that warps rarely take), and V = (M << 96) >> R with
// R = 208 - T + S - E, at least 18 because S > E; V is read from an 8-word
// frame by a three-level word select and one funnel shift per word.  Zeros,
// infinities, NaNs and empty rows (S = kOzakiScaleEmpty) give V = 0.
template <int NW>
QB_HD void crt_scaled_words(q128 a, int S, int T, uint32_t (&w)[NW], bool& neg) {
  neg = (a.hi >> 63) != 0;
  const int be = (int)((a.hi >> 48) & 0x7FFFu);
  uint64_t mh = a.hi & kMantHiMask, ml = a.lo;
  int E = be - kBias;
  bool zero = be == kExpField || S == kOzakiScaleEmpty;
  if (be != 0) {
    mh |= kHiddenBit;
  } else if ((mh | ml) == 0) {
    zero = true;
  } else {
    q_unpack_norm(a, mh, ml, E);
  }
  int R = 208 - T + S - E;
  R = zero ? 255 : (R < 0 ? 0 : (R > 255 ? 255 : R));
  const uint32_t k = (uint32_t)R >> 5, b = (uint32_t)R & 31u;
  const uint32_t x[16] = {0u, 0u, 0u, (uint32_t)ml, (uint32_t)(ml >> 32), (uint32_t)mh, (uint32_t)(mh >> 32), 0u,
                          0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
  uint32_t z[NW + 4], u[NW + 2], y[NW + 1];
#pragma unroll
  for (int j = 0; j < NW + 4; ++j) z[j] = (k & 4u) ? x[j + 4] : x[j];
#pragma unroll
  for (int j = 0; j < NW + 2; ++j) u[j] = (k & 2u) ? z[j + 2] : z[j];
#pragma unroll
  for (int j = 0; j < NW + 1; ++j) y[j] = (k & 1u) ? u[j + 1] : u[j];
#pragma unroll
  for (int i = 0; i < NW; ++i) w[i] = fshr32(y[i], y[i + 1], b);
}

// fp16 bits of an integer |v| <= 2048 (exact)
inline uint16_t crt_half_bits(int v) {
  if (v == 0) return 0;
  const uint16_t sign = v < 0 ? 0x8000u : 0u;
  uint32_t a = (uint32_t)(v < 0 ? -v : v);
  int e = 0;
  while ((a >> e) > 1) ++e;  // a in [2^e, 2^(e+1))
  const uint32_t frac = (a << (10 - e)) & 0x3FFu;
  return (uint16_t)(sign | ((uint32_t)(e + 15) << 10) | frac);
}

inline int crt_balanced(int64_t v, uint32_t p) {
  int64_t r = v % (int64_t)p;
  if (r < 0) r += p;
  if (r > (int64_t)(p / 2)) r -= p;
  return (int)r;
}

inline void crt_split_table(const CrtTable& tab, CrtSplitTable& st) {
  st = CrtSplitTable();
  st.nmod = tab.n;
  st.T = tab.T;
  st.NB = tab.T <= 144 ? 18 : 24;
  st.N = 2 * ((tab.n + 7) / 8 * 8);
  for (int q = 0; q < tab.n; ++q) {
    const uint32_t p = tab.mod[q].p;
    st.p[q] = (float)p;
    st.inv_p[q] = (float)(1.0 / (double)p);
    uint32_t ib, nb;
    const float np = -(float)p;
    memcpy(&ib, &st.inv_p[q], 4);
    memcpy(&nb, &np, 4);
    st.inv_p2[q] = ((uint64_t)ib << 32) | ib;
    st.neg_p2[q] = ((uint64_t)nb << 32) | nb;
  }
  for (int n = 0; n < st.N; ++n) {
    const int q = n / 2, e = n % 2;
    int64_t csum = 0;
    int c[32] = {0};
    if (q < tab.n) {
      const uint32_t p = tab.mod[q].p;
      int64_t pw = 1 % p;
      for (int j = 0; j < st.NB; ++j) {
        c[j] = crt_balanced(pw, p);
        csum += c[j];
        pw = pw * 256 % p;
      }
      c[st.NB] = crt_balanced(1024 * csum, p);
    }
    for (int k = 0; k < kCrtSplitK; ++k) {
      const int ek = k / 32, j = k % 32;
      const int v = (q < tab.n && ek == e && j <= st.NB) ? c[j] : 0;
      st.b[(k / 8) * (st.N * 8) + n * 8 + (k % 8)] = crt_half_bits(v);
    }
  }
}

// ---------------------------------------------------------------------------
// Residues and reconstruction (host and device)
// ---------------------------------------------------------------------------
// x mod p for x < 2^31: with magic = ceil(2^40 / p) = (2^40 + e) / p,
// 0 <= e < p <= 513, x magic / 2^40 = x / p + x e / (p 2^40) and x e < 2^40,
// so the floor is floor(x / p).
QB_HD uint32_t crt_mod(uint32_t x, uint32_t p, uint32_t magic) {
#if defined(__CUDA_ARCH__)
  const uint32_t q = __umulhi(x, magic) >> 8;
#else
  const uint32_t q = (uint32_t)(((uint64_t)x * magic) >> 40);
#endif
  return x - q * p;
}

// The 18-bit pieces of V = (v2:v1:v0), least significant first (NP = 8
// covers T <= 144, 11 covers T <= 198); the shifts are constants once the
// loop is unrolled.
template <int NP>
QB_HD void crt_pieces(uint64_t v0, uint64_t v1, uint64_t v2, uint32_t (&h)[NP]) {
#pragma unroll
  for (int j = 0; j < NP; ++j) {
    const int b = 18 * j, w = b >> 6, o = b & 63;
    uint64_t x = (w == 0 ? v0 : (w == 1 ? v1 : v2)) >> o;
    if (o > 46 && w < 2) x |= (w == 0 ? v1 : v2) << (64 - o);
    h[j] = (uint32_t)x & 0x3FFFFu;
  }
}

// The balanced residue r == V (mod p), |r| <= floor(p/2) <= 256, of V with
// pieces h, plus floor(p/2): (V + floor(p/2)) mod p, from
// x = floor(p/2) + sum_j h_j (2^(18 j) mod p) < 256 + 11 * 2^18 * 512 < 2^31.
template <int NP>
QB_HD uint32_t crt_residue_shifted(const uint32_t (&h)[NP], const CrtMod& m) {
  uint32_t x = m.half;
#pragma unroll
  for (int j = 0; j < NP; ++j) x += h[j] * m.c18[j];
  return crt_mod(x, m.p, m.magic);
}

template <int NP>
QB_HD int crt_residue(const uint32_t (&h)[NP], const CrtMod& m) {
  return (int)crt_residue_shifted<NP>(h, m) - (int)m.half;
}

// The N balanced residues of a (sign included) for row scale S, T bits.
QB_HD void crt_residues(q128 a, int S, const CrtTable& tab, int* r) {
  uint64_t v0, v1, v2;
  bool neg;
  ozaki_scaled_bits(a, S, tab.T, v0, v1, v2, neg);
  uint32_t h[kCrtPieces];
  crt_pieces<kCrtPieces>(v0, v1, v2, h);
  for (int q = 0; q < tab.n; ++q) {
    const int x = crt_residue<kCrtPieces>(h, tab.mod[q]);
    r[q] = neg ? -x : x;
  }
}

// C_q mod p for |C_q| <= 2^29 (one pass), and y_q = (C_q mod p) u_q mod p.
QB_HD uint32_t crt_reduce(int32_t c, const CrtMod& m) {
  return crt_mod((uint32_t)(c + (int32_t)m.K), m.p, m.magic);
}
QB_HD uint32_t crt_y(uint32_t r, const CrtMod& m) { return crt_mod(r * m.u, m.p, m.magic); }

// Reconstruction accumulators of one output: Y = sum_q y_q M / p_q by 32-bit
// word position (each word sum stays below 2^57), and sum_q y_q round(2^24 /
// p_q), whose rounding to a multiple of 2^24 is Q (its error is below
// 48 * 513 * 2^-25 < 2^-10 units of 2^24, and |X / M| < 1/8).
template <int NW>
struct CrtAcc {
  uint64_t a[NW];
  uint32_t q;
};

template <int NW>
QB_HD void crt_acc_init(CrtAcc<NW>& A) {
#pragma unroll
  for (int w = 0; w < NW; ++w) A.a[w] = 0;
  A.q = 0;
}

// Adds moduli p0 and p1 (residue terms y0, y1) with W = M / (p0 p1):
// y0 M / p0 + y1 M / p1 = (y0 p1 + y1 p0) W.  A last unpaired modulus is
// passed with y1 = 0, p1 = 1, P1 = 0 and W = M / p0.
template <int NW>
QB_HD void crt_acc_pair(CrtAcc<NW>& A, uint32_t y0, uint32_t y1, uint32_t p0, uint32_t p1, uint32_t P0,
                        uint32_t P1, const uint32_t* W) {
  A.q += y0 * P0 + y1 * P1;
  const uint32_t z = y0 * p1 + y1 * p0;  // < 2 * 513^2 < 2^20
#pragma unroll
  for (int w = 0; w < NW; ++w) A.a[w] += (uint64_t)z * W[w];
}

// Word i of X, zero outside [0, NW) (i a constant once inlined).
template <int NW>
QB_HD uint32_t crt_word_at(const uint32_t (&X)[NW], int i) {
  return (i >= 0 && i < NW) ? X[(i >= 0 && i < NW) ? i : 0] : 0u;
}

// The five words X[k], X[k-1], ..., X[k-4] (zero below word 0): one branch
// per value of k, each reading fixed registers (the outputs of a warp mostly
// share k, so a warp mostly takes one branch).
template <int NW>
QB_HD void crt_window5(const uint32_t (&X)[NW], int k, uint32_t& h4, uint32_t& h3, uint32_t& h2, uint32_t& h1,
                       uint32_t& h0) {
  static_assert(NW <= 12, "at most 12 words");
#define QB_CRT_WINDOW_CASE(K)                                                                        \
  case K:                                                                                           \
    h4 = crt_word_at<NW>(X, K);                                                                     \
    h3 = crt_word_at<NW>(X, K - 1);                                                                 \
    h2 = crt_word_at<NW>(X, K - 2);                                                                 \
    h1 = crt_word_at<NW>(X, K - 3);                                                                 \
    h0 = crt_word_at<NW>(X, K - 4);                                                                 \
    break;
  switch (k) {
    QB_CRT_WINDOW_CASE(11)
    QB_CRT_WINDOW_CASE(10)
    QB_CRT_WINDOW_CASE(9)
    QB_CRT_WINDOW_CASE(8)
    QB_CRT_WINDOW_CASE(7)
    QB_CRT_WINDOW_CASE(6)
    QB_CRT_WINDOW_CASE(5)
    QB_CRT_WINDOW_CASE(4)
    QB_CRT_WINDOW_CASE(3)
    QB_CRT_WINDOW_CASE(2)
    QB_CRT_WINDOW_CASE(1)
    default:
      QB_CRT_WINDOW_CASE(0)
  }
#undef QB_CRT_WINDOW_CASE
}

// X 2^e rounded to binary128 (RNE), X in two's complement over NW words.
// The magnitude's highest nonzero word k (from a mask of the nonzero words)
// gives a window of five words, normalised by one count of leading zeros:
// the significand's 113 bits, the round bit and the sticky bits are fixed
// positions of it; the words below the window count only as sticky bits
// (the mask again).  Results below the normal range or above it take the
// general rounding (round_pack).
template <int NW>
QB_HD q128 crt_round_x(uint32_t (&X)[NW], int e) {
  static_assert(NW % 2 == 0 && NW >= 8, "reconstruction of 8, 10 or 12 words");
  const uint32_t neg = X[NW - 1] >> 31, mask = 0u - neg;
  {
    uint64_t c = neg;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      c += (uint32_t)(X[w] ^ mask);
      X[w] = (uint32_t)c;
      c >>= 32;
    }
  }
  uint32_t nz = 0;
#pragma unroll
  for (int w = 0; w < NW; ++w) nz |= (X[w] != 0u ? 1u : 0u) << w;
  if (nz == 0) return q_zero(neg);
  const int k = 31 - clz32(nz);
  uint32_t h4, h3, h2, h1, h0;
  crt_window5<NW>(X, k, h4, h3, h2, h1, h0);
  const bool below = k >= 5 && (nz & ((1u << (k - 4)) - 1u)) != 0u;
  const int lz = clz32(h4);
  // the window shifted left by lz: its top bit is X's leading one
  const uint32_t g4 = fshl32_any(h3, h4, lz), g3 = fshl32_any(h2, h3, lz), g2 = fshl32_any(h1, h2, lz),
                 g1 = fshl32_any(h0, h1, lz), g0 = h0 << lz;
  const int E = e + 32 * k + 31 - lz;  // exponent of the leading one
  const int be = E + kBias;
  if (be <= 0 || be >= kExpField) {  // subnormal or overflowing result: the general rounding
    uint64_t V[NW / 2];
#pragma unroll
    for (int i = 0; i < NW / 2; ++i) V[i] = (uint64_t)X[2 * i] | ((uint64_t)X[2 * i + 1] << 32);
    u256 m = u256_make(V[3], V[2], V[1], V[0]);
    int drop = 0;
#pragma unroll
    for (int d = 1; d <= NW / 2 - 4; ++d)
      if (V[3 + d] != 0) {
        m = u256_make(V[3 + d], V[2 + d], V[1 + d], V[d]);
        drop = d;
      }
    bool sticky = false;
#pragma unroll
    for (int i = 0; i < NW / 2 - 4; ++i) sticky = sticky || (i < drop && V[i] != 0);
    return round_pack(neg, m, sticky, e + 64 * drop);
  }
  // significand: g4, g3, g2 and the top 17 bits of g1; round bit: bit 14 of g1
  uint64_t rh = ((uint64_t)g4 << 17) | (g3 >> 15);
  uint64_t rl = ((uint64_t)((g3 << 17) | (g2 >> 15)) << 32) | (uint32_t)((g2 << 17) | (g1 >> 15));
  const bool rbit = (g1 >> 14) & 1u;
  const bool st = below || (g1 & 0x3FFFu) != 0 || g0 != 0;
  int bexp = be;
  if (rbit && (st || (rl & 1))) {
    rl += 1;
    if (rl == 0) rh += 1;
    if (rh >> 49) {  // carried into bit 113: the significand is 2^113
      rh >>= 1;
      bexp += 1;
      if (bexp >= kExpField) return q_inf(neg);
    }
  }
  return make_q(((uint64_t)neg << 63) | ((uint64_t)bexp << 48) | (rh & kMantHiMask), rl);
}

// X = Y - Q M (two's complement modulo 2^(32 NW); |X| < (32/65) M), and
// X 2^e rounded to binary128 (RNE).
template <int NW>
QB_HD q128 crt_acc_round(const CrtAcc<NW>& A, const uint32_t* negM, int e) {
  const uint64_t Q = (A.q + (1u << 23)) >> 24;
  uint32_t X[NW];
  uint64_t c = 0;
#pragma unroll
  for (int w = 0; w < NW; ++w) {
    c += A.a[w] + Q * negM[w];
    X[w] = (uint32_t)c;
    c >>= 32;
  }
  return crt_round_x<NW>(X, e);
}

// ---------------------------------------------------------------------------
// Reconstruction on the tensor cores: the table (host) and the column sums
// ---------------------------------------------------------------------------
// Y = sum_q y_q M / p_q with M / p_q = sum_w W_qw 256^w (bytes) is
// Y = sum_w Z_w 256^w, Z_w = sum_q y_q W_qw: a product of the reduced
// residues y (one MMA operand row per output, fp16, y <= 512) and the bytes
// W (fp16) with Z_w <= 48 * 512 * 255 < 2^23, exact in fp32.  Two more
// columns carry the bytes of P24_q = round(2^24 / p_q) (< 2^16), whose sums
// give Q as crt_acc_round does.  nbytes = 4 NW - 1 bytes hold M / p_q <
// 2^(32 NW) / 257.  Columns: bytes 0 .. nbytes-1, then P24's low and high
// byte; N = nbytes + 2 rounded up to 16.
// MMA width of the reconstruction for NW words: nbytes + 2 columns rounded
// up to 16.
QB_HD constexpr int crt_fold_n(int NW) { return (4 * NW + 1 + 15) / 16 * 16; }

constexpr int kCrtFoldK = kCrtMaxMods;  // 48: K of the MMA (moduli, zero beyond nmod)
constexpr int kCrtFoldMaxN = 64;

struct alignas(16) CrtFoldTable {
  int nmod, N, nbytes, nw;
  uint32_t negM[kCrtMaxWords];
  uint32_t p[kCrtMaxMods], magic[kCrtMaxMods];
  // B (N rows, K = modulus) in the shared-memory layout of a K-major operand
  // without swizzle: the 16 bytes of (row n, k-block kb) at kb * (N * 16) + n * 16
  uint16_t b[kCrtFoldK * kCrtFoldMaxN];
};

inline void crt_fold_table(const CrtTable& tab, CrtFoldTable& ft) {
  ft = CrtFoldTable();
  ft.nmod = tab.n;
  ft.nw = tab.nw;
  ft.nbytes = 4 * tab.nw - 1;
  ft.N = crt_fold_n(tab.nw);
  for (int w = 0; w < kCrtMaxWords; ++w) ft.negM[w] = tab.negM[w];
  for (int q = 0; q < tab.n; ++q) {
    ft.p[q] = tab.mod[q].p;
    ft.magic[q] = tab.mod[q].magic;
  }
  for (int q = 0; q < tab.n; ++q) {
    uint32_t Mq[kCrtMaxWords + 2] = {1};
    for (int r = 0; r < tab.n; ++r)
      if (r != q) crt_big_mul_small(Mq, kCrtMaxWords + 2, tab.mod[r].p);
    for (int n = 0; n < ft.N; ++n) {
      int v = 0;
      if (n < ft.nbytes)
        v = (int)((Mq[n / 4] >> (8 * (n % 4))) & 0xFFu);
      else if (n == ft.nbytes)
        v = (int)(tab.mod[q].P24 & 0xFFu);
      else if (n == ft.nbytes + 1)
        v = (int)(tab.mod[q].P24 >> 8);
      ft.b[(q / 8) * (ft.N * 8) + n * 8 + (q % 8)] = crt_half_bits(v);
    }
  }
}

// The reconstruction from the column sums, one column at a time (w a
// constant once unrolled): byte columns w < nbytes = 4 NW - 1 go into the
// sum of their word, T_(w/4) += Z_w 256^(w mod 4) (each word's sum its own,
// below 2^49, so that no carry chain runs through the columns), the two
// columns after them make S = sum_q y_q P24_q; then Q, and one carry pass
// over the words gives X = Y - Q M = sum_w (T_w + Q (2^(32 NW) - M)_w) 2^(32 w)
// (mod 2^(32 NW)), which is rounded at 2^e.
template <int NW>
struct CrtFoldAcc {
  uint64_t T[NW];  // word sums (with the columns' offsets when biased)
  uint32_t S;
};

template <int NW>
QB_HD void crt_fold_init(CrtFoldAcc<NW>& A) {
  A.S = 0;
#pragma unroll
  for (int i = 0; i < NW; ++i) A.T[i] = 0;
}

// t + (uint64_t)a * b in one wide multiply-add
QB_HD uint64_t crt_mad_wide(uint32_t a, uint32_t b, uint64_t t) {
#if defined(__CUDA_ARCH__)
  uint64_t r;
  asm("mad.wide.u32 %0, %1, %2, %3;" : "=l"(r) : "r"(a), "r"(b), "l"(t));
  return r;
#else
  return t + (uint64_t)a * b;
#endif
}

// Byte column w with sum z.  bias != 0: z is given as 2^23 + z (the bits of
// the fp32 value z + 2^23) and the 2^23 of each column is taken off once per
// word.
template <int NW>
QB_HD void crt_fold_column(CrtFoldAcc<NW>& A, int w, uint32_t z, bool bias = false) {
  constexpr int nbytes = 4 * NW - 1;
  if (w < nbytes) {
    A.T[w >> 2] = crt_mad_wide(z, 1u << (8 * (w & 3)), A.T[w >> 2]);
  } else if (w == nbytes) {
    A.S += bias ? z - 0x4B000000u : z;
  } else if (w == nbytes + 1) {
    A.S += (bias ? z - 0x4B000000u : z) << 8;
  }
}

template <int NW>
QB_HD q128 crt_fold_finish(CrtFoldAcc<NW>& A, const uint32_t* negM, int e, bool bias = false) {
  const uint32_t Q = (A.S + (1u << 23)) >> 24;  // below 2^8
  // T_w + Q negM_w for every word at once (T_w < 2^49 once its offsets are
  // off, Q negM_w < 2^40), then the carries
  uint64_t V[NW];
#pragma unroll
  for (int w = 0; w < NW; ++w) {
    // the last word holds three columns (bytes 4 NW - 4 .. 4 NW - 2)
    const uint64_t off = bias ? 0x4B000000ull * (w == NW - 1 ? 0x00010101ull : 0x01010101ull) : 0ull;
    V[w] = crt_mad_wide(Q, negM[w], A.T[w] - off);
  }
  uint32_t X[NW];
  uint64_t c = 0;
#pragma unroll
  for (int w = 0; w < NW; ++w) {
    c += V[w];
    X[w] = (uint32_t)c;
    c >>= 32;
  }
  return crt_round_x<NW>(X, e);
}

// All columns at once (host form): Z[0 .. nbytes + 1].
template <int NW>
QB_HD q128 crt_fold_columns(const uint32_t* Z, int nbytes, const uint32_t* negM, int e) {
  CrtFoldAcc<NW> A;
  crt_fold_init(A);
  for (int w = 0; w < nbytes + 2; ++w) crt_fold_column(A, w, Z[w]);
  return crt_fold_finish(A, negM, e);
}

// Host and test form: the binary128 value of X 2^e for the residue sums
// C_q (one pass, |C_q| <= 2^29) of one output.
template <int NW>
QB_HD q128 crt_reconstruct(const int32_t* C, const CrtTable& tab, int e) {
  CrtAcc<NW> A;
  crt_acc_init(A);
  for (int i = 0; 2 * i < tab.n; ++i) {
    const CrtMod& m0 = tab.mod[2 * i];
    const uint32_t y0 = crt_y(crt_reduce(C[2 * i], m0), m0);
    if (2 * i + 1 < tab.n) {
      const CrtMod& m1 = tab.mod[2 * i + 1];
      const uint32_t y1 = crt_y(crt_reduce(C[2 * i + 1], m1), m1);
      crt_acc_pair(A, y0, y1, m0.p, m1.p, m0.P24, m1.P24, tab.Mpair[i]);
    } else {
      crt_acc_pair(A, y0, 0u, m0.p, 1u, m0.P24, 0u, tab.Mpair[i]);
    }
  }
  return crt_acc_round(A, tab.negM, e);
}

QB_HD q128 crt_reconstruct_any(const int32_t* C, const CrtTable& tab, int e) {
  if (tab.nw <= 8) return crt_reconstruct<8>(C, tab, e);
  if (tab.nw <= 10) return crt_reconstruct<10>(C, tab, e);
  return crt_reconstruct<12>(C, tab, e);
}

}  // namespace qb
