"""The oracle pinned against the reference: committed golden fixtures made
by the reference itself (tests/golden), the reference compiled here when
its tree is present (oracle/_ref), the reference's known answers, and an
independent exact-rational check of the long accumulator."""
import os
from fractions import Fraction

import numpy as np
import pytest

from qblas_gb300 import gen as G
from qblas_gb300 import quad as Q

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_outputs.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLDEN)


def test_golden_dot(O, gold):
    for name in ("dot_small", "dot_par", "dot_strided", "dot_strided_small"):
        n, incx, incy, T = (int(v) for v in gold[f"{name}_meta"])
        got = O.ref_dot(gold[f"{name}_x"], gold[f"{name}_y"], n, incx, incy, T)
        assert Q.same_bits(got, gold[f"{name}_out"]).all(), name


def test_golden_axpy(O, gold):
    got = O.ref_axpy(Q.scalar(2.5), gold["axpy_x"], gold["axpy_y"], nthreads=4)
    assert Q.same_bits(got, gold["axpy_out"]).all()


def test_golden_gemv(O, gold):
    for tag in ("gemv_row", "gemv_col"):
        cm, m, n, lda = (int(v) for v in gold[f"{tag}_meta"])
        got = O.ref_gemv(cm, m, n, Q.scalar(1.5), gold[f"{tag}_A"], lda, gold[f"{tag}_x"], 1, Q.scalar(0.5),
                         gold[f"{tag}_y"], 1, lib_order=1, nthreads=4)
        assert Q.same_bits(got, gold[f"{tag}_out"]).all(), tag


def test_golden_gemm(O, gold):
    for tag in ("gemm_simple", "gemm_blocked"):
        m, n, k = (int(v) for v in gold[f"{tag}_meta"])
        got = O.ref_gemm(0, m, n, k, Q.scalar(2.5), gold[f"{tag}_A"], k, gold[f"{tag}_B"], n, Q.scalar(1.5),
                         gold[f"{tag}_C"], n, lib_order=1, nthreads=4)
        assert Q.same_bits(got, gold[f"{tag}_out"]).all(), tag


def test_golden_kats(O, gold):
    kat = dict(zip([str(s) for s in gold["kat_names"]], gold["kat_values"]))
    # test_quadblas.cpp:205-224 (55), :715-739 (1e20 + 1 - 1e20 = 1), :290-312 (norm of 1..1000)
    assert kat["dot_1_to_10"] == 55.0
    assert kat["dot_1e20_cancel"] == 1.0
    x = Q.from_double(np.arange(1, 11))
    assert O.to_double(O.ref_dot(x, Q.from_double(np.ones(10))))[0] == 55.0
    R, r, _ = O.exact_dot(Q.from_double([1e20, 1.0, -1e20]), Q.from_double([1.0, 1.0, 1.0]))
    assert O.to_double(R)[0] == 1.0 and Q.same_bits(r, Q.scalar(0.0)).all()
    x = Q.from_double(np.arange(1, 1001))
    R, _, _ = O.exact_dot(x, x)
    nrm = O.to_double(O.sqrt(R))[0]
    assert nrm == kat["nrm2_1_to_1000"]
    assert abs(nrm - np.sqrt(1000 * 1001 * 2001 / 6)) < 1e-12 * np.sqrt(1000)


def test_reference_tree_matches_restatement(O):
    """Run where the reference tree was compiled (oracle/_ref)."""
    import ctypes
    R = O.ref_lib()
    if R is None:
        pytest.skip("oracle/_ref not built (reference tree absent)")
    rng = G.rng_for(11)
    c64, cint, P = ctypes.c_int64, ctypes.c_int, O.P
    for n, incx, incy, T in [(499, 1, 1, 3), (500, 1, 1, 3), (3001, 1, 1, 7), (900, 2, 5, 3)]:
        x, y = G.uniform_full(rng, n * incx), G.uniform_full(rng, n * incy)
        a = O.qs(1)
        R.qref_dot(c64(n), P(x), c64(incx), P(y), c64(incy), cint(T), P(a))
        assert Q.same_bits(a, O.ref_dot(x, y, n, incx, incy, T)).all()
    for cm in (0, 1):
        m, n = 37, 91
        lda = n + 3 if cm == 0 else m + 2
        A = G.uniform_full(rng, (m if cm == 0 else n) * lda)
        x, y = G.uniform_full(rng, n * 2), G.uniform_full(rng, m)
        al, be = Q.scalar(-0.75), Q.scalar(3.0)
        yr = y.copy()
        R.qref_gemv(cint(cm), c64(m), c64(n), P(al), P(A), c64(lda), P(x), c64(2), P(be), P(yr), c64(1), cint(2))
        assert Q.same_bits(yr, O.ref_gemv(cm, m, n, al, A, lda, x, 2, be, y, 1, lib_order=1, nthreads=2)).all()
    for (m, n, k) in [(65, 9, 131), (5, 70, 3), (64, 64, 64)]:
        A, B, C = G.uniform_full(rng, m * k), G.uniform_full(rng, k * n), G.uniform_full(rng, m * n)
        al, be = Q.scalar(2.5), Q.scalar(-1.5)
        Cr = C.copy()
        R.qref_gemm(cint(0), c64(m), c64(n), c64(k), P(al), P(A), c64(k), P(B), c64(n), P(be), P(Cr), c64(n),
                    cint(4))
        assert Q.same_bits(Cr, O.ref_gemm(0, m, n, k, al, A, k, B, n, be, C, n, lib_order=1, nthreads=4)).all()


# ---- independent check of the exact accumulator with Python rationals -----
def q_to_fraction(w) -> Fraction:
    lo, hi = int(w[0]), int(w[1])
    sign = -1 if hi >> 63 else 1
    be = (hi >> 48) & 0x7FFF
    mant = ((hi & ((1 << 48) - 1)) << 64) | lo
    assert be != 0x7FFF
    if be == 0:
        return sign * Fraction(mant) * Fraction(2) ** (-16382 - 112)
    return sign * Fraction(mant | (1 << 112)) * Fraction(2) ** (be - 16383 - 112)


def fraction_to_q(F: Fraction):
    """Round an exact rational to binary128, ties to even."""
    if F == 0:
        return (0, 0)
    sign = 1 if F < 0 else 0
    F = abs(F)
    e = F.numerator.bit_length() - F.denominator.bit_length()
    if Fraction(2) ** e > F:
        e -= 1
    lsb = max(e - 112, -16494)
    scaled = F / Fraction(2) ** lsb
    R = scaled.numerator // scaled.denominator
    rem = scaled - R
    if rem > Fraction(1, 2) or (rem == Fraction(1, 2) and R & 1):
        R += 1
    if R >> 113:
        R >>= 1
        lsb += 1
    if R >> 112:
        be = lsb + 112 + 16383
        assert be < 0x7FFF
        hi = (sign << 63) | (be << 48) | ((R >> 64) & ((1 << 48) - 1))
    else:
        hi = (sign << 63) | (R >> 64)
    return (R & ((1 << 64) - 1), hi)


def test_exact_accumulator_vs_rationals(O):
    import quadvec as V
    rng = G.rng_for(5)
    for t in range(40):
        n = int(rng.integers(1, 60))
        kind = t % 4
        if kind == 0:
            x, y = G.uniform_full(rng, n), G.uniform_full(rng, n)
        elif kind == 1:
            x, y = G.cancelling_dot(rng, max(n, 4), -200, 200)
        elif kind == 2:
            x, y = V.finite(rng, n, -16382, -16300), V.finite(rng, n, -100, 10)
        else:
            x, y = V.finite(rng, n, -3, 3, sparse=True), V.finite(rng, n, -3, 3, sparse=True)
        S = sum((q_to_fraction(a) * q_to_fraction(b) for a, b in zip(x, y)), Fraction(0))
        R, r, _ = O.exact_dot(x, y)
        assert tuple(int(v) for v in R[0]) == fraction_to_q(S), (t, kind)
        if S != 0:
            assert tuple(int(v) for v in r[0]) == fraction_to_q(S - q_to_fraction(R[0])), (t, kind)


def test_exact_accumulator_order_invariant(O):
    rng = G.rng_for(9)
    x, y = G.cancelling_dot(rng, 5000)
    R1, r1, _ = O.exact_dot(x, y)
    p = rng.permutation(5000)
    R2, r2, _ = O.exact_dot(x[p], y[p])
    assert Q.same_bits(R1, R2).all() and Q.same_bits(r1, r2).all()
    # x.y + (-x).y == 0 exactly
    xn = x.copy()
    xn[:, 1] ^= np.uint64(1 << 63)
    R3, _, _ = O.exact_dot(np.concatenate([x, xn]), np.concatenate([y, y]))
    assert Q.same_bits(R3, Q.scalar(0.0)).all()


def test_exact_accumulator_negative_totals(O):
    # a negative running total survives many intermediate roundings (GenDot
    # rounds the accumulator once per generated pair)
    rng = G.rng_for(13)
    x, y = G.cancelling_dot(rng, 4000, -100, 100)
    R, r, _ = O.exact_dot(x, y)
    xn = x.copy()
    xn[:, 1] ^= np.uint64(1 << 63)
    Rn, rn, _ = O.exact_dot(xn, y)
    for a, b in ((Rn, R), (rn, r)):
        neg = b.copy()
        neg[:, 1] ^= np.uint64(1 << 63)
        assert Q.same_bits(a, neg).all()


@pytest.mark.parametrize("cond", [1e10, 1e20, 1e30, 1e40])
def test_gendot_condition(O, cond):
    x, y = O.gendot(4096, cond, 7)
    c = O.dot_condition(x, y)
    assert cond / 10 <= c <= cond * 1e3, c
    x2, y2 = O.gendot(4096, cond, 7)
    assert Q.same_bits(x, x2).all() and Q.same_bits(y, y2).all()
