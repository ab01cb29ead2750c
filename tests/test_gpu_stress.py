"""Ill-conditioned accuracy stress on GenDot inputs (dot products of
prescribed condition, Ogita-Rump-Oishi), against the exact oracle.

* qdot, k = 8192, condition 1e10, 1e20, 1e30, 1e40 (three seeds each).
* qgemm, m = n = 2048, k = 8192: row i of A and column i of B form a GenDot
  pair whose condition cycles through the four values, so the diagonal
  C(i, i) carries the prescribed condition; 2048 off-diagonal entries are
  checked as well.  Soft-float, then Ozaki with 15 digits of 9 bits, 17 and
  20 of 8 bits and 22 of 7 bits.

Bounds asserted (u_q = 2^-113, ulps of the exact result):
  * soft-float: correctly rounded (<= 0.5 ulp) at every condition (the
    wide accumulator's rounding is certified, and sums that cancel below
    its 256-bit frame are recomputed exactly), hence also within
    k * u_q * sum|a_i b_i|.
  * Ozaki with s digits of b bits: |error| <= k (s + 3) 2^(Sa + Sb - b s)
    + 1 ulp, where 2^Sa, 2^Sb bound the row of A and the column of B (the
    split keeps each element to 2^(S - b s + 1) and drops the digit pairs
    t + u >= s, each at most 2^(2(b-1)) 2^(Sa + Sb - 2(b-1) - b(t+u))).
The max-ulp and max-relative errors per condition are printed and, when
QBLAS_STRESS_REPORT names a file, written there as JSON.
"""
import json
import os

import numpy as np
import pytest

from qblas_gb300 import api
from qblas_gb300 import quad as Q

pytestmark = pytest.mark.gpu

CONDS = (1e10, 1e20, 1e30, 1e40)
K = 8192
MN = 2048
REPORT = {}


@pytest.fixture(scope="module", autouse=True)
def report():
    yield REPORT
    path = os.environ.get("QBLAS_STRESS_REPORT")
    print("\nGenDot stress (max ulp / max relative error vs the exact oracle):")
    for key in sorted(REPORT):
        print(f"  {key}: {REPORT[key]}")
    if path:
        with open(path, "w") as f:
            json.dump(REPORT, f, indent=1, sort_keys=True)


def exponents(a):
    """Unbiased exponent of each binary128 value (normal values)."""
    a = Q.as_quad(a)
    return ((a[:, 1] >> np.uint64(48)) & np.uint64(0x7FFF)).astype(np.int64) - 16383


def errors(O, got, R, r):
    """(ulps of R, relative error) of each result."""
    ulp = O.ulp_err(got, R, r)
    ulp_size = np.exp2((exponents(R) - 112).astype(np.float64))
    rel = ulp * ulp_size / np.abs(O.to_double(R))
    return ulp, rel


def summary(ulp, rel):
    return {"max_ulp": float(np.max(ulp)), "max_rel": float(np.max(rel))}


def test_qdot_gendot(qlib, O):
    api.set_method(0)
    for cond in CONDS:
        ulps, rels = [], []
        for seed in (1, 2, 3):
            x, y = O.gendot(K, cond, seed)
            got = api.dot(x, y)
            R, r, ab = O.exact_dot(x, y)
            u, rl = errors(O, got, R, r)
            ulps.append(u[0])
            rels.append(rl[0])
            assert O.bound_violations(got, R, ab, K) == 0, (cond, seed)
            assert u[0] <= 0.5, (cond, seed, u[0])
        REPORT[f"qdot k=8192 cond={cond:.0e} softfloat"] = summary(np.array(ulps), np.array(rels))


@pytest.fixture(scope="module")
def gendot_matrices(O):
    conds = np.array([CONDS[i % 4] for i in range(MN)])
    X, Y = O.gendot_batch(K, conds, np.arange(MN, dtype=np.uint64) + 1000)
    A = X  # row i of A (m x k, row-major) is x^(i)
    B = np.ascontiguousarray(Y.reshape(MN, K, 2).transpose(1, 0, 2)).reshape(-1, 2)  # B[:, j] = y^(j)
    rng = np.random.default_rng(5)
    rows = np.concatenate([np.arange(MN), rng.integers(0, MN, MN)])
    cols = np.concatenate([np.arange(MN), rng.integers(0, MN, MN)])
    off = rows != cols
    R, r, ab = O.exact_gemm(K, A, K, 1, B, MN, 1, rows, cols, nthreads=os.cpu_count() or 8)
    ea = exponents(A).reshape(MN, K).max(axis=1) + 1  # |A(i, l)| < 2^Sa_i
    eb = exponents(Y).reshape(MN, K).max(axis=1) + 1  # |B(l, j)| < 2^Sb_j
    return dict(A=A, B=B, rows=rows, cols=cols, off=off, R=R, r=r, ab=ab, conds=conds, Sa=ea, Sb=eb)


def run_gemm(M):
    C = np.zeros((MN * MN, 2), dtype=np.uint64)
    api.gemm("R", "N", "N", MN, MN, K, Q.scalar(1.0), M["A"], K, M["B"], MN, Q.scalar(0.0), C, MN)
    return C[M["rows"] * MN + M["cols"]]


def record(O, M, label, got):
    ulp, rel = errors(O, got, M["R"], M["r"])
    diag = ~M["off"]
    for c in CONDS:
        sel = diag & (M["conds"][M["rows"]] == c)
        REPORT[f"qgemm 2048x2048x8192 cond={c:.0e} {label}"] = summary(ulp[sel], rel[sel])
    REPORT[f"qgemm 2048x2048x8192 off-diagonal {label}"] = summary(ulp[M["off"]], rel[M["off"]])
    return ulp


def test_qgemm_gendot_softfloat(qlib, O, gendot_matrices):
    M = gendot_matrices
    api.set_method(0)
    got = run_gemm(M)
    ulp = record(O, M, "softfloat", got)
    assert O.bound_violations(got, M["R"], M["ab"], K) == 0
    assert ulp.max() <= 0.5


@pytest.mark.parametrize("s,b,scheme", [(15, 9, 1), (17, 8, 1), (20, 8, 1), (22, 7, 1), (15, 9, 2), (22, 7, 2)])
def test_qgemm_gendot_ozaki(qlib, O, gendot_matrices, s, b, scheme):
    """Both Ozaki schemes truncate the operands to b*s - 1 bits; the residue
    scheme (2) has no further error, the digit pairs (1) drop the pairs below
    the digit count."""
    M = gendot_matrices
    api.set_method(2)
    api.set_ozaki_slices(s)
    api.set_ozaki_digit_bits(b)
    api.set_ozaki_scheme(scheme)
    try:
        got = run_gemm(M)
    finally:
        api.set_method(0)
        api.set_ozaki_slices(0)
        api.set_ozaki_digit_bits(0)
        api.set_ozaki_scheme(0)
    label = f"ozaki s={s} b={b}" + (" residues" if scheme == 2 else "")
    ulp = record(O, M, label, got)
    # normwise bound of the split, in log2, with the final rounding's ulp
    err_log2 = np.log2(np.maximum(ulp, 1e-300)) + (exponents(M["R"]) - 112)
    Sab = M["Sa"][M["rows"]] + M["Sb"][M["cols"]]
    bound_log2 = np.log2(K * (s + 3)) + Sab - b * s
    within = (ulp <= 1.0) | (err_log2 <= bound_log2 + 1e-9)
    assert within.all(), np.argwhere(~within)[:5]
