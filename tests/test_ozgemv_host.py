"""The Ozaki qgemv arithmetic (qblas_gb300/csrc/ozgemv.cuh, compiled for the
host) against exact rationals:

* window: W - R = floor(|a| / 2^(E - 141)) < 2^142, and the 18 balanced
  digits reconstruct it, each in [-128, 128) (a's digits carry its sign);
* chunk: the diagonal sums stay below 2^24 (exact in fp32), T is
  sum_{g<20} D_g 256^(19-g), and |T 2^(E+F-162) - sum_j a_j x_j| < 2^(E+F-133);
* row: every certified rounding equals the correctly rounded exact sum (the
  exact oracle), and wide-exponent rows are almost all certified;
* partition: the CTAs' item ranges tile [0, work) in order and og_cta_of
  names the range that holds each item (row partials are written and read
  by that index).
"""
import ctypes
from fractions import Fraction

import numpy as np
import pytest

from qblas_gb300 import gen as G
from qblas_gb300 import quad as Q
from test_oracle import q_to_fraction

R_WINDOW = sum(128 << (8 * t) for t in range(18))


def P(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def lead_top(w):
    be = (int(w[1]) >> 48) & 0x7FFF
    return (be if be else 1) - 16383


def windows(sq, a, E):
    a = np.ascontiguousarray(a)
    E = np.ascontiguousarray(np.asarray(E, dtype=np.int32))
    W = np.zeros((len(a), 5), dtype=np.uint32)
    sq.sq_og_window(ctypes.c_int64(len(a)), P(a), P(E), P(W))
    return [sum(int(w[k]) << (32 * k) for k in range(5)) for w in W]


def sample(rng, n):
    parts = [G.wide_exponent(rng, n), G.uniform_full(rng, n), G.spread_uniform(rng, n, -300, 300)]
    sub = G.uniform_full(rng, n)
    sub[:, 1] &= ~np.uint64(0x7FFF << 48)  # subnormals
    zero = np.zeros((n // 4 + 1, 2), dtype=np.uint64)
    zero[::2, 1] = np.uint64(1 << 63)
    return np.concatenate(parts + [sub, zero])


def test_window_digits(sq):
    rng = G.rng_for(91)
    a = sample(rng, 400)
    leads = np.array([lead_top(w) for w in a])
    E = leads + rng.integers(0, 170, size=len(a))
    for w, e, W in zip(a, E, windows(sq, a, E)):
        assert W < 1 << 144
        V = W - R_WINDOW
        f = q_to_fraction(w)
        exact = abs(f) / Fraction(2) ** (int(e) - 141)
        mag = exact.numerator // exact.denominator
        assert V == mag, (w, e)
        assert V < 1 << 142
        d = [((W >> (8 * (17 - t))) & 0xFF) - 128 for t in range(18)]
        assert all(-128 <= x < 128 for x in d)
        assert sum(x << (8 * (17 - t)) for t, x in enumerate(d)) == V


def test_window_short_form(sq):
    """The kernel's short window (no four-word shift level) equals the general
    one whenever the shift is below 128."""
    rng = G.rng_for(95)
    a = sample(rng, 400)
    leads = np.array([lead_top(w) for w in a])
    E = np.ascontiguousarray((leads + rng.integers(0, 125, size=len(a))).astype(np.int32))
    W = np.zeros((len(a), 5), dtype=np.uint32)
    sq.sq_og_window_short(ctypes.c_int64(len(a)), P(np.ascontiguousarray(a)), P(E), P(W))
    full = windows(sq, a, E)
    for i, w in enumerate(W):
        if int(w[0]) == 0xFFFFFFFF and int(w[4]) == 0xFFFFFFFF:
            continue  # shift of 128 or more (zeros and subnormals against a large E)
        assert sum(int(w[k]) << (32 * k) for k in range(5)) == full[i], i


def chunk(sq, a, x):
    EF = np.zeros(2, dtype=np.int32)
    D = np.zeros(32, dtype=np.int64)
    T = np.zeros(6, dtype=np.uint32)
    sq.sq_og_chunk(ctypes.c_int(len(a)), P(np.ascontiguousarray(a)), P(np.ascontiguousarray(x)), P(EF), P(D), P(T))
    t = sum(int(T[k]) << (32 * k) for k in range(6))
    if t >> 191:
        t -= 1 << 192
    return int(EF[0]), int(EF[1]), D, t


@pytest.mark.parametrize("kind", ["wide", "uniform", "spread", "extreme"])
def test_chunk_bound(sq, kind):
    rng = G.rng_for(92)
    for trial in range(40):
        n = 32 if trial % 5 else int(rng.integers(1, 32))
        if kind == "wide":
            a, x = G.wide_exponent(rng, n), G.wide_exponent(rng, n)
        elif kind == "uniform":
            a, x = G.uniform_full(rng, n), G.uniform_full(rng, n)
        elif kind == "spread":
            a, x = G.spread_uniform(rng, n, -2000, 2000), G.spread_uniform(rng, n, -40, 40)
        else:  # every significand all ones: digit sums at their largest
            a, x = G.uniform_full(rng, n), G.uniform_full(rng, n)
            a[:, 0] = x[:, 0] = np.uint64(0xFFFFFFFFFFFFFFFF)
            a[:, 1] |= np.uint64(0xFFFFFFFFFFFF)
            x[:, 1] |= np.uint64(0xFFFFFFFFFFFF)
            a[:, 1] = (a[:, 1] & ~np.uint64(0x7FFF << 48)) | np.uint64(16383 << 48)
            x[:, 1] = (x[:, 1] & ~np.uint64(0x7FFF << 48)) | np.uint64(16383 << 48)
        E, F, D, T = chunk(sq, a, x)
        assert np.all(np.abs(D) < 1 << 24)
        assert T == sum(int(D[g]) << (8 * (19 - g)) for g in range(20))
        exact = sum(q_to_fraction(u) * q_to_fraction(v) for u, v in zip(a, x))
        approx = Fraction(T) * Fraction(2) ** (E + F - 162)
        assert abs(approx - exact) < Fraction(2) ** (E + F - 133), (kind, trial)


def row(sq, a, x):
    out = np.zeros((1, 2), dtype=np.uint64)
    ok = sq.sq_og_row(ctypes.c_int64(len(a)), P(np.ascontiguousarray(a)), P(np.ascontiguousarray(x)), P(out))
    return ok, out


@pytest.mark.parametrize("kind,n,min_rate", [("wide", 1000, 0.95), ("uniform", 777, 0.95),
                                             ("cancel", 512, 0.0)])
def test_row_certified_is_exact(sq, O, kind, n, min_rate):
    rng = G.rng_for(93)
    rows, certified = 40, 0
    for r in range(rows):
        if kind == "wide":
            a, x = G.wide_exponent(rng, n), G.wide_exponent(rng, n)
        elif kind == "uniform":
            a, x = G.uniform_full(rng, n), G.uniform_full(rng, n)
        else:
            a, x = G.cancelling_dot(rng, n)
        ok, out = row(sq, a, x)
        R, _, _ = O.exact_dot(a, x)
        if ok:
            certified += 1
            assert Q.same_bits(out, R).all(), (kind, r)
    assert certified >= min_rate * rows, certified


def test_row_zeros_and_specials(sq, O):
    rng = G.rng_for(94)
    a, x = G.uniform_full(rng, 100), np.zeros((100, 2), dtype=np.uint64)
    ok, out = row(sq, a, x)  # x all zero: every product is an exact zero
    assert ok and Q.same_bits(out, Q.scalar(0.0)).all()
    a[7] = Q.as_quad(np.array([[0, 0x7FFF << 48]], dtype=np.uint64))[0]  # +inf in the row
    ok, _ = row(sq, a, G.uniform_full(rng, 100))
    assert not ok


@pytest.mark.parametrize("work,G", [(1, 1), (5, 5), (7, 3), (16384, 152), (1000, 152), (152, 152),
                                    (153, 152), (64 * 257, 152), (12345, 97)])
def test_work_partition(sq, work, G):
    begin = np.zeros(G + 1, dtype=np.int64)
    cta = np.zeros(work, dtype=np.int64)
    sq.sq_og_partition(ctypes.c_int64(work), ctypes.c_int64(G), P(begin), P(cta))
    assert begin[0] == 0 and begin[G] == work and np.all(np.diff(begin) >= 0)
    want = np.searchsorted(begin, np.arange(work), side="right") - 1
    assert np.array_equal(cta, want)
