"""The Ozaki digit split and fold (ozaki.cuh, compiled for the host) against
an independent restatement in Python integers: for each element the scaled
integer V = trunc(|a| 2^(b*s - 1 - S)) is cut into balanced base-2^b digits
from the least significant end (centred remainders, the top digit takes the
rest), and the fold sum_g C_g 2^(b(G-g)) is rounded once; plus the
representation bound |a - sum_t d_t 2^(S-(b-1)-b t)| < 2^(S - b s + 1)."""
from fractions import Fraction

import numpy as np
import pytest

import ozaki_emul as E
import quadvec as V
from qblas_gb300 import gen as G
from test_oracle import fraction_to_q, q_to_fraction


def digits_py(w, S, s, b):
    lo, hi = int(w[0]), int(w[1])
    neg = hi >> 63
    be = (hi >> 48) & 0x7FFF
    mant = ((hi & ((1 << 48) - 1)) << 64) | lo
    if be == 0x7FFF or (be == 0 and mant == 0) or S == -(1 << 29):
        return [0] * s
    if be == 0:
        e = -16382 - 112 + mant.bit_length() - 1
        m = mant << (113 - mant.bit_length())
    else:
        m, e = mant | (1 << 112), be - 16383
    sh = e + b * s - 113 - S
    v = m << sh if sh >= 0 else m >> (-sh)
    d = []
    for _ in range(s - 1):
        r = v & ((1 << b) - 1)
        if r >= 1 << (b - 1):
            r -= 1 << b
        d.append(r)
        v = (v - r) >> b
    d.append(v)
    d = d[::-1]
    return [-x for x in d] if neg else d


@pytest.mark.parametrize("b,s", [(7, 2), (7, 13), (7, 20), (7, 22), (8, 2), (8, 11), (8, 17), (8, 20),
                                 (9, 2), (9, 15), (9, 18)])
def test_digits_match_integer_restatement(sq, b, s):
    rng = G.rng_for(100 * b + s)
    X = np.concatenate([G.spread_uniform(rng, 160), V.finite(rng, 40, -16382, -16300), V.subnormal(rng, 40),
                        G.wide_exponent(rng, 40, -300, 300), np.zeros((16, 2), np.uint64)])
    rows, cols = 4, len(X) // 4
    S, D = E.split(sq, X, rows, cols, cols, 1, s, b)
    assert np.abs(D).max() <= 1 << (b - 1)
    for r in range(rows):
        for c in range(cols):
            ref = digits_py(X[r * cols + c], int(S[r]), s, b)
            assert [int(D[t, r, c]) for t in range(s)] == ref, (r, c)
            x = q_to_fraction(X[r * cols + c])
            rec = sum(Fraction(int(D[t, r, c])) * Fraction(2) ** (int(S[r]) - (b - 1) - b * t) for t in range(s))
            assert abs(x - rec) < Fraction(2) ** (int(S[r]) - b * s + 1)


@pytest.mark.parametrize("b", [7, 8, 9])
def test_fold_matches_integer_restatement(sq, b):
    rng = np.random.default_rng(b)
    s, m, n = 17, 5, 6
    C = rng.integers(-(2**31) + 1, 2**31 - 1, size=(s, m, n), dtype=np.int64)
    Sa = rng.integers(-40, 40, size=m).astype(np.int32)
    Fb = rng.integers(-40, 40, size=n).astype(np.int32)
    out = E.fold(sq, C, Sa, Fb, b)
    G_ = s - 1
    for i in range(m):
        for j in range(n):
            R = sum(int(C[g, i, j]) << (b * (G_ - g)) for g in range(s))
            e = int(Sa[i]) + int(Fb[j]) - 2 * (b - 1) - b * G_
            exp = fraction_to_q(Fraction(R) * Fraction(2) ** e)
            assert (int(out[i * n + j][0]), int(out[i * n + j][1])) == exp
