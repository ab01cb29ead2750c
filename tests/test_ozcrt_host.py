"""The Ozaki scheme II arithmetic (qblas_gb300/csrc/ozcrt.cuh, compiled for
the host) against Python integers and rationals:

* table: pairwise coprime moduli whose product M exceeds (65/32) k 2^(2T)
  (and the shortest such prefix), the inverses (M/p)^-1 mod p, M / (p p') per
  pair, 2^(32 nw) - M and the 2^(18 j) mod p tables;
* crt_mod: the magic-multiplier remainder equals x % p for x < 2^31;
* residues: V = trunc(|a| 2^(T - S)) and balanced residues r == sign * V
  (mod p), |r| <= 256;
* reconstruction: from C_q == X (mod p_q), |C_q| <= 2^29, the result is X 2^e
  correctly rounded (ties to even), for X across (-(32/65) M, (32/65) M),
  the range k 2^(2T) < (32/65) M allows.
"""
import ctypes
import math
from fractions import Fraction

import numpy as np
import pytest

from qblas_gb300 import gen as G
from test_oracle import fraction_to_q, q_to_fraction

MAXMODS, MAXWORDS, PIECES = 48, 12, 11
TABLE_WORDS = 4 + MAXMODS * (2 + PIECES) + (MAXMODS // 2) * MAXWORDS + MAXWORDS


def P(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def words(ws):
    return sum(int(w) << (32 * i) for i, w in enumerate(ws))


def table(sq, T, k):
    out = np.zeros(TABLE_WORDS, dtype=np.uint32)
    n = sq.sq_crt_table(ctypes.c_int(T), ctypes.c_int64(k), P(out))
    if n == 0:
        return None
    nw = int(out[1])
    o = 4
    mods = []
    for q in range(MAXMODS):
        p, u = int(out[o]), int(out[o + 1])
        mods.append((p, u, [int(c) for c in out[o + 2:o + 2 + PIECES]]))
        o += 2 + PIECES
    mpair = [words(out[o + i * MAXWORDS:o + (i + 1) * MAXWORDS]) for i in range(MAXMODS // 2)]
    o += (MAXMODS // 2) * MAXWORDS
    negm = words(out[o:o + MAXWORDS])
    return n, nw, mods[:n], mpair, negm


CASES = [(134, 4096), (143, 4096), (143, 1 << 20), (118, 64), (161, 8192), (80, 1), (170, 1 << 30)]


@pytest.mark.parametrize("T,k", CASES)
def test_table(sq, T, k):
    t = table(sq, T, k)
    assert t is not None
    n, nw, mods, mpair, negm = t
    ps = [m[0] for m in mods]
    assert all(256 < p <= 513 for p in ps)
    assert all(math.gcd(a, b) == 1 for i, a in enumerate(ps) for b in ps[i + 1:])
    M = math.prod(ps)
    need = 65 * k << (2 * T)
    assert 32 * M > need and 32 * math.prod(ps[:-1]) <= need
    assert M < 1 << (32 * nw) and nw % 2 == 0 and nw <= MAXWORDS
    for p, u, c18 in mods:
        assert (M // p) * u % p == 1
        assert c18 == [pow(2, 18 * j, p) for j in range(PIECES)]
    for i in range(0, n, 2):
        div = ps[i] * (ps[i + 1] if i + 1 < n else 1)
        assert mpair[i // 2] == M // div
    assert negm == (1 << (32 * nw)) - M


def test_table_limits(sq):
    assert table(sq, 192, 16) is None       # more bits than the split's three 64-bit words hold
    assert table(sq, 191, 1 << 40) is None  # more moduli than the table holds


def test_table_covers_every_digit_setting(sq):
    """The automatic scheme takes residues for every digit count the library
    accepts: 2..22 digits of 7 bits, 2..20 of 8, 2..18 of 9 (T <= 161), for k
    up to 2^31 - 1; at most 41 moduli and 12 words are needed."""
    for bits, smax in ((7, 22), (8, 20), (9, 18)):
        for s in range(2, smax + 1):
            for k in (1, 64, 4096, 1 << 20, (1 << 31) - 1):
                t = table(sq, bits * s - 1, k)
                assert t is not None, (bits, s, k)
                assert t[0] <= 41 and t[1] <= MAXWORDS, (bits, s, k, t[0], t[1])


def test_crt_mod(sq):
    rng = np.random.default_rng(7)
    x = np.concatenate([rng.integers(0, 1 << 31, 20000, dtype=np.uint64),
                        np.arange(0, 5000, dtype=np.uint64),
                        (1 << 31) - 1 - np.arange(0, 5000, dtype=np.uint64)]).astype(np.uint32)
    for p in [513, 512, 511, 509, 505, 257, 263, 269, 277, 281, 283, 293, 307, 311, 317]:
        r = np.zeros_like(x)
        sq.sq_crt_mod(ctypes.c_int64(len(x)), P(x), ctypes.c_uint32(p), P(r))
        assert np.array_equal(r, x % np.uint32(p)), p


def lead_exp(w):
    f = q_to_fraction(w)
    if f == 0:
        return None
    e = abs(f).numerator.bit_length() - abs(f).denominator.bit_length()
    return e if Fraction(2) ** e <= abs(f) else e - 1


@pytest.mark.parametrize("T", [134, 143, 161])
def test_residues(sq, T):
    rng = G.rng_for(301)
    a = np.concatenate([G.wide_exponent(rng, 300), G.uniform_full(rng, 300),
                        G.spread_uniform(rng, 300, -400, 400), np.zeros((4, 2), dtype=np.uint64)])
    a[-1, 1] = np.uint64(1 << 63)  # -0
    sub = G.uniform_full(rng, 20)
    sub[:, 1] &= ~np.uint64(0x7FFF << 48)
    a = np.ascontiguousarray(np.concatenate([a, sub]))
    S = []
    for w in a:
        e = lead_exp(w)
        S.append(-(1 << 29) if e is None else e + 1 + int(rng.integers(0, 60)))
    S = np.array(S, dtype=np.int32)
    k = 4096
    n, _, mods, _, _ = table(sq, T, k)
    r = np.zeros((len(a), n), dtype=np.int32)
    V = np.zeros((len(a), 4), dtype=np.uint64)
    assert sq.sq_crt_residues(ctypes.c_int64(len(a)), P(a), P(S), ctypes.c_int(T), ctypes.c_int64(k), P(r), P(V)) == n
    for i, w in enumerate(a):
        v = int(V[i, 0]) | (int(V[i, 1]) << 64) | (int(V[i, 2]) << 128)
        f = abs(q_to_fraction(w))
        if S[i] == -(1 << 29):
            assert v == 0
        else:
            exact = f * Fraction(2) ** (T - int(S[i]))
            assert v == exact.numerator // exact.denominator and v < 1 << T
        sv = -v if V[i, 3] else v
        for q, (p, _, _) in enumerate(mods):
            assert abs(int(r[i, q])) <= 256
            assert (int(r[i, q]) - sv) % p == 0


def test_reconstruct(sq):
    T, k = 134, 4096
    n, nw, mods, _, _ = table(sq, T, k)
    ps = [m[0] for m in mods]
    M = math.prod(ps)
    rng = np.random.default_rng(11)
    Xs = [0, 1, -1, 2, (1 << 113) - 1, -(1 << 113) + 1, (1 << 114) + 1, (1 << 114) + 3, -((1 << 114) + 3),
          (1 << 200) + (1 << 87), (1 << 200) + (1 << 87) + 1, M // 8 - 1, -(M // 8) + 1,
          k << (2 * T), -(k << (2 * T)), (k << (2 * T)) - 1, -(k << (2 * T)) + 1,
          32 * M // 65 - 1, -(32 * M // 65) + 1, 32 * M // 65 - 12345, -(32 * M // 65) + 98765]
    for b in range(1, M.bit_length(), 7):
        x = int(rng.integers(0, 1 << 62)) << max(0, b - 62)
        x = x % (1 << b) | (1 << (b - 1))
        Xs += [x, -x]
    Xs = [x for x in Xs if 65 * abs(x) < 32 * M]
    C = np.zeros((len(Xs), n), dtype=np.int32)
    for i, x in enumerate(Xs):
        for q, p in enumerate(ps):
            c = x % p + p * int(rng.integers(-(1 << 29) // p, (1 << 29) // p - 1))
            assert abs(c) <= 1 << 29
            C[i, q] = c
    e = rng.integers(-300, 100, size=len(Xs)).astype(np.int32)
    out = np.zeros((len(Xs), 2), dtype=np.uint64)
    assert sq.sq_crt_reconstruct(ctypes.c_int64(len(Xs)), P(C), P(e), ctypes.c_int(T), ctypes.c_int64(k), P(out)) == n
    for i, x in enumerate(Xs):
        want = fraction_to_q(Fraction(x) * Fraction(2) ** int(e[i]))
        assert (int(out[i, 0]), int(out[i, 1])) == want, (i, x)


def test_reconstruct_all_word_counts(sq):
    """8, 10 and 12 words (small T, the bench's T, large T)."""
    rng = np.random.default_rng(12)
    for T, k in [(100, 64), (134, 4096), (170, 1 << 20)]:
        n, nw, mods, _, _ = table(sq, T, k)
        ps = [m[0] for m in mods]
        X = [int(rng.integers(1, 1 << 62)) << int(rng.integers(0, 2 * T - 62)) for _ in range(50)]
        X = [x if j % 2 else -x for j, x in enumerate(X)]
        C = np.array([[x % p for p in ps] for x in X], dtype=np.int32)
        e = np.full(len(X), -2 * T, dtype=np.int32)
        out = np.zeros((len(X), 2), dtype=np.uint64)
        sq.sq_crt_reconstruct(ctypes.c_int64(len(X)), P(C), P(e), ctypes.c_int(T), ctypes.c_int64(k), P(out))
        for i, x in enumerate(X):
            assert (int(out[i, 0]), int(out[i, 1])) == fraction_to_q(Fraction(x, 1 << (2 * T))), (T, nw, i)


def scaled(f, S, T):
    """sign * trunc(|f| 2^(T - S)) as a Python integer."""
    v = abs(f) * Fraction(2) ** (T - S)
    v = v.numerator // v.denominator
    return -v if f < 0 else v


def row_scale(ws):
    es = [lead_exp(w) for w in ws]
    es = [e for e in es if e is not None]
    return max(es) + 1 if es else -(1 << 29)


@pytest.mark.parametrize("T,k", [(134, 40), (143, 33), (71, 17), (161, 9000)])
def test_crt_gemm_emulation_exact(sq, T, k):
    """Host residues + exact residue products + host reconstruction equal the
    correctly rounded exact sum of the T-bit truncated products."""
    import ozaki_emul as E
    rng = G.rng_for(302 + T)
    m, n = (3, 2) if k > 1000 else (5, 4)
    A = G.spread_uniform(rng, m * k, -30, 30)
    B = G.spread_uniform(rng, k * n, -30, 30)
    A[1 * k:2 * k] = 0  # an all-zero row
    got = E.crt_gemm_sum(sq, m, n, k, A, k, 1, B, n, 1, T)
    fa = [[q_to_fraction(A[i * k + l]) for l in range(k)] for i in range(m)]
    fb = [[q_to_fraction(B[l * n + j]) for l in range(k)] for j in range(n)]
    S = [row_scale(A[i * k:(i + 1) * k]) for i in range(m)]
    F = [row_scale(B[j::n]) for j in range(n)]
    for i in range(m):
        for j in range(n):
            if S[i] == -(1 << 29) or F[j] == -(1 << 29):
                want = (0, 0)
            else:
                X = sum(scaled(fa[i][l], S[i], T) * scaled(fb[j][l], F[j], T) for l in range(k))
                want = fraction_to_q(Fraction(X) * Fraction(2) ** (S[i] + F[j] - 2 * T))
            assert (int(got[i * n + j, 0]), int(got[i * n + j, 1])) == want, (i, j)



def half_to_int(h):
    """Integer value of fp16 bit patterns that hold integers (|v| <= 2048)."""
    h = h.astype(np.int64)
    e = (h >> 10) & 0x1F
    m = (h & 0x3FF) | 0x400
    v = np.where(e == 0, 0, np.where(e >= 25, m << np.maximum(e - 25, 0), m >> np.maximum(25 - e, 0)))
    return np.where(h & 0x8000, -v, v)


@pytest.mark.parametrize("T,k", [(134, 4096), (143, 4096), (161, 8192), (180, 64)])
def test_tensor_core_split(sq, T, k):
    """The residue split as the tensor cores compute it (ozaki_crt_split_tc_kernel):
    the operand row of an element (fp16 s(1024 + b_j) for the NB bytes of V,
    then -s) times the table's B must be an integer below 2^24 (exact in the
    fp32 accumulation) congruent to s V modulo each p, and the fp32 rounding
    r = x - p round(x fl(1/p)) (emulated exactly with integers: fl(1/p) = M
    2^E, the fused multiply-add with 1.5 * 2^23 rounds to the nearest integer,
    ties to even) must give the balanced residue, |r| <= 256."""
    head = np.zeros(4, dtype=np.int32)
    pb = np.zeros(MAXMODS, dtype=np.uint32)
    ib = np.zeros(MAXMODS, dtype=np.uint32)
    b = np.zeros(64 * 2 * MAXMODS, dtype=np.uint16)
    n = sq.sq_crt_split_table(ctypes.c_int(T), ctypes.c_int64(k), P(head), P(pb), P(ib), P(b))
    assert n > 0
    nmod, N, NB, TT = (int(v) for v in head)
    assert nmod == n and TT == T and NB == (18 if T <= 144 else 24) and N % 16 == 0 and 2 * n <= N < 2 * n + 16
    # B[k][col] from the shared-memory layout: (k-block, row n, k % 8)
    B = np.zeros((64, N), dtype=np.int64)
    for kk in range(64):
        for col in range(N):
            B[kk, col] = half_to_int(np.array([b[(kk // 8) * (N * 8) + col * 8 + kk % 8]]))[0]
    p = pb[:n].view(np.float32).astype(np.int64)
    # V: random T-bit integers, edge values, both signs
    rng = np.random.default_rng(T)
    cnt = 3000
    Vs = [int(rng.integers(0, 1 << 62)) | (int(rng.integers(0, 1 << 62)) << 62) | (int(rng.integers(0, 1 << 62)) << 124)
          for _ in range(cnt)]
    Vs = [v & ((1 << T) - 1) for v in Vs] + [0, (1 << T) - 1, 1, 1 << (T - 1), int("80" * 24, 16) & ((1 << T) - 1)]
    signs = [int(rng.integers(0, 2)) for _ in Vs[:-5]] + [1, 0, 1, 0, 1]
    A = np.zeros((len(Vs), 64), dtype=np.int64)
    for i, (v, s) in enumerate(zip(Vs, signs)):
        sg = -1 if s else 1
        for j in range(NB):
            A[i, j] = sg * (1024 + ((v >> (8 * j)) & 0xFF))
        A[i, NB] = -sg
    A[:-1, 32:] = A[1:, :32]  # the second element of each row: the next value
    X = A @ B
    assert np.abs(X).max() < 1 << 23
    assert not X[:, 2 * n:].any()  # padding columns
    for e in (0, 1):
        x = X[:-1, e::2][:, :n]
        vs, sgs = (Vs[:-1], signs[:-1]) if e == 0 else (Vs[1:], signs[1:])
        for q in range(n):
            bits = int(ib[q])
            M = (bits & 0x7FFFFF) | 0x800000
            E = ((bits >> 23) & 0xFF) - 127 - 23  # 1/p = M 2^E
            sh = -E
            t = x[:, q] * M  # x / p ~= t / 2^sh, |t| < 2^47
            qf = t >> sh
            rem = t - (qf << sh)
            half = 1 << (sh - 1)
            qq = qf + ((rem > half) | ((rem == half) & (qf & 1 == 1))).astype(np.int64)
            r = x[:, q] - qq * p[q]
            assert np.abs(r).max() <= 256, (T, q, int(p[q]))
            for i, (v, s) in enumerate(zip(vs, sgs)):
                sv = -v if s else v
                assert (int(r[i]) - sv) % int(p[q]) == 0


@pytest.mark.parametrize("T", [98, 134, 143, 180])
def test_scaled_words_match_scaled_bits(sq, T):
    """The split kernel's branch-free scaling (crt_scaled_words) gives the
    same V and sign as ozaki_scaled_bits for normal, subnormal, zero, -0,
    infinite and NaN elements, and scales from just above the element's
    exponent to far beyond it (V = 0)."""
    rng = G.rng_for(700 + T)
    a = np.concatenate([G.wide_exponent(rng, 2000), G.spread_uniform(rng, 2000, -400, 400),
                        np.zeros((4, 2), dtype=np.uint64)])
    sub = G.uniform_full(rng, 200)
    sub[:, 1] &= ~np.uint64(0x7FFF << 48)
    sub[:100, 1] &= np.uint64(0x8000000000000000)  # subnormals whose leading one is in the low word
    spec = np.zeros((3, 2), dtype=np.uint64)
    spec[0, 1] = np.uint64(0x7FFF << 48)  # +inf
    spec[1, 1] = np.uint64(0xFFFF << 48)  # -inf
    spec[2, 1] = np.uint64(0x7FFF8 << 44)  # NaN
    a = np.ascontiguousarray(np.concatenate([a, sub, spec]))
    a[2005, 1] = np.uint64(1 << 63)  # -0
    S = []
    for w in a:
        special = (int(w[1]) >> 48) & 0x7FFF == 0x7FFF
        e = None if special else lead_exp(w)
        r = int(rng.integers(0, 4))
        if e is None:
            S.append(-(1 << 29) if r == 0 else int(rng.integers(-100, 100)))
        else:
            S.append(e + 1 + [0, 1, int(rng.integers(0, 200)), int(rng.integers(0, 20000))][r])
    S = np.array(S, dtype=np.int32)
    S[:7] = -(1 << 29)  # empty rows
    out = np.zeros((len(a), 7), dtype=np.uint32)
    ref = np.zeros((len(a), 4), dtype=np.uint64)
    sq.sq_crt_scaled_words(ctypes.c_int64(len(a)), P(a), P(S), ctypes.c_int(T), P(out), P(ref))
    for i in range(len(a)):
        v = sum(int(out[i, j]) << (32 * j) for j in range(6))
        r = int(ref[i, 0]) | (int(ref[i, 1]) << 64) | (int(ref[i, 2]) << 128)
        assert v == r, (i, hex(v), hex(r))
        if r:
            assert out[i, 6] == ref[i, 3]


@pytest.mark.parametrize("T,k", [(100, 64), (134, 4096), (143, 4096), (170, 1 << 20)])
def test_tensor_core_reconstruction(sq, T, k):
    """The reconstruction as the tensor cores compute it (ozaki_crt_fold_tc_kernel):
    column sums of the reduced residues times the bytes of M / p_q (and of
    round(2^24 / p_q)) from the fp16 table, assembled with carries, equal
    X 2^e correctly rounded, and every column sum stays below 2^23 (exact in
    the fp32 accumulation and in the 2^23 conversion)."""
    n, nw, mods, _, _ = table(sq, T, k)
    ps = [m[0] for m in mods]
    M = math.prod(ps)
    rng = np.random.default_rng(T + 5)
    Xs = [0, 1, -1, M // 8 - 1, -(M // 8) + 1]
    for _ in range(300):
        b = int(rng.integers(1, M.bit_length() - 4))
        x = (int(rng.integers(0, 1 << 62)) << max(0, b - 62)) % (1 << b) | (1 << (b - 1))
        Xs.append(x if rng.integers(2) else -x)
    Xs = [x for x in Xs if 65 * abs(x) < 32 * M]
    C = np.zeros((len(Xs), n), dtype=np.int32)
    for i, x in enumerate(Xs):
        for q, p in enumerate(ps):
            C[i, q] = x % p + p * int(rng.integers(-(1 << 29) // p, (1 << 29) // p - 1))
    e = rng.integers(-2 * T - 50, -2 * T + 50, size=len(Xs)).astype(np.int32)
    out = np.zeros((len(Xs), 2), dtype=np.uint64)
    ref = np.zeros((len(Xs), 2), dtype=np.uint64)
    zmax = ctypes.c_int64(0)
    assert sq.sq_crt_fold_tc(ctypes.c_int64(len(Xs)), P(C), P(e), ctypes.c_int(T), ctypes.c_int64(k), P(out),
                             ctypes.byref(zmax)) == n
    sq.sq_crt_reconstruct(ctypes.c_int64(len(Xs)), P(C), P(e), ctypes.c_int(T), ctypes.c_int64(k), P(ref))
    assert 0 < zmax.value < 1 << 23
    assert (out == ref).all()
    for i, x in enumerate(Xs):
        assert (int(out[i, 0]), int(out[i, 1])) == fraction_to_q(Fraction(x) * Fraction(2) ** int(e[i])), (i, x)


def test_reconstruct_rounding_edges(sq):
    """The reconstruction's rounding of X 2^e: ties (even and odd), sticky
    bits far below, carries into a new binade, subnormal and overflowing
    results (the general path), against exact rational rounding."""
    T, k = 134, 4096
    n, nw, mods, _, _ = table(sq, T, k)
    ps = [m[0] for m in mods]
    M = math.prod(ps)
    rng = np.random.default_rng(99)
    cases = []
    for top in (113, 114, 120, 150, 200, 250):
        base = 1 << (top - 1)
        cases += [base, base + 1, base | ((1 << (top - 113)) - 1), (1 << top) - 1,
                  base + (1 << (top - 114)) if top > 113 else base,                  # tie, even
                  base + (1 << (top - 113)) + (1 << (top - 114)) if top > 113 else base,  # tie, odd
                  base + (1 << (top - 114)) + 1 if top > 114 else base]
    for _ in range(200):
        top = int(rng.integers(1, M.bit_length() - 4))
        cases.append(int(rng.integers(1, 1 << 62)) << max(0, top - 62) | 1)
    cases = [c for c in cases if 0 < c < M // 8]
    Xs, es = [], []
    for c in cases:
        for sgn in (1, -1):
            for e in (-2 * T, -2 * T - 16400, -2 * T + 16000, 0):
                Xs.append(sgn * c)
                es.append(e)
    keep = []
    for x, e in zip(Xs, es):
        f = Fraction(x) * Fraction(2) ** e
        if abs(f) < Fraction(2) ** 16384 * (1 - Fraction(1, 2 ** 114)):  # below the overflow threshold
            keep.append((x, e))
    C = np.array([[x % p for p in ps] for x, _ in keep], dtype=np.int32)
    e = np.array([e for _, e in keep], dtype=np.int32)
    out = np.zeros((len(keep), 2), dtype=np.uint64)
    sq.sq_crt_reconstruct(ctypes.c_int64(len(keep)), P(C), P(e), ctypes.c_int(T), ctypes.c_int64(k), P(out))
    for i, (x, ee) in enumerate(keep):
        assert (int(out[i, 0]), int(out[i, 1])) == fraction_to_q(Fraction(x) * Fraction(2) ** ee), (i, x, ee)


@pytest.mark.parametrize("k", [4096, 7600])
@pytest.mark.parametrize("sign", [1, -1])
def test_crt_gemm_largest_sums(sq, k, sign):
    """Every operand 1 - 2^-113 (significand all ones) and every product of
    one sign: X = k (2^134 - 2^21)^2, the largest sum T = 134 bits allow.
    For k = 7600 the 32 moduli still cover it and |X| = 0.4917 M, next to the
    32/65 M the quotient estimate is proved for (k = 4096: 0.265 M)."""
    import ozaki_emul as E
    T, m, n = 134, 2, 3
    n_mod, _, _, _, _ = table(sq, T, k)
    assert n_mod == 32
    top = np.array([0xFFFFFFFFFFFFFFFF, 0x3FFEFFFFFFFFFFFF], dtype=np.uint64)  # 1 - 2^-113
    A = np.tile(top, (m * k, 1))
    B = np.tile(top, (k * n, 1))
    if sign < 0:
        B[:, 1] |= np.uint64(1 << 63)
    got = E.crt_gemm_sum(sq, m, n, k, A, k, 1, B, n, 1, T)
    want = fraction_to_q(sign * k * (1 - Fraction(1, 1 << 113)) ** 2)
    assert all((int(g[0]), int(g[1])) == want for g in got)
