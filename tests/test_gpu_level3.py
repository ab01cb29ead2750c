"""GPU parity of the soft-float qgemm against the oracle, through the C ABI.

Tolerance: each C(i,j) must be bit-identical to
fma(alpha, R_ij, beta*C_ij) with R_ij the correctly rounded exact sum
(exact long accumulator); against the reference's own per-k-panel FMA
chains it must stay within (k + 2) * u_q * (|alpha| sum|a b| + |beta c|).
"""
import os

import numpy as np
import pytest

from conftest import to_dev, to_host
from gpu_helpers import epilogue, epilogue_bound
from qblas_gb300 import api
from qblas_gb300 import gen as G
from qblas_gb300 import quad as Q

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_outputs.npz")


def strides(layout, transa, transb, lda, ldb, ldc):
    col = layout in "Cc"
    ta, tb = transa in "TtCc", transb in "TtCc"
    if not col:
        sa = (1, lda) if ta else (lda, 1)
        sb = (1, ldb) if tb else (ldb, 1)
        sc = (ldc, 1)
    else:
        sa = (lda, 1) if ta else (1, lda)
        sb = (ldb, 1) if tb else (1, ldb)
        sc = (1, ldc)
    return sa, sb, sc


def expected_entries(O, layout, transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, rows, cols):
    (sai, sal), (sbl, sbj), (sci, scj) = strides(layout, transa, transb, lda, ldb, ldc)
    R, _, ab = O.exact_gemm(k, A, sai, sal, B, sbl, sbj, rows, cols, nthreads=16)
    idx = rows * sci + cols * scj
    return idx, epilogue(O, alpha, R, beta, C[idx]), ab


def test_gemm_known_answers(qlib):
    # test_quadblas.cpp:447-464: [[1,2],[3,4]] @ [[5,6],[7,8]] = [[19,22],[43,50]]
    A, B = Q.from_double([1, 2, 3, 4]), Q.from_double([5, 6, 7, 8])
    C = Q.from_double(np.zeros(4))
    api.qgemm("R", "N", "N", 2, 2, 2, 1.0, A, 2, B, 2, 0.0, C, 2)
    assert np.array_equal(Q.to_double_approx(C), [19, 22, 43, 50])
    # :679-688: 1x1 3*4 = 12
    C1 = Q.from_double([0.0])
    api.qgemm("R", "N", "N", 1, 1, 1, 1.0, Q.from_double([3.0]), 1, Q.from_double([4.0]), 1, 0.0, C1, 1)
    assert Q.to_double_approx(C1)[0] == 12.0
    # :691-712: I @ A = A exactly
    n = 50
    rng = G.rng_for(1)
    Aq = G.uniform_full(rng, n * n)
    I = Q.from_double(np.eye(n).ravel())
    C = Q.from_double(np.zeros(n * n))
    api.qgemm("R", "N", "N", n, n, n, 1.0, I, n, Aq, n, 0.0, C, n)
    assert Q.same_bits(C, Aq).all()


SHAPES = [(1, 1, 1), (2, 3, 4), (47, 31, 23), (33, 65, 17), (64, 64, 64), (65, 66, 67), (130, 70, 300)]


@pytest.mark.parametrize("layout", ["R", "C"])
@pytest.mark.parametrize("trans", ["NN", "TN", "NT", "TT"])
def test_gemm_bit_exact(qlib, O, layout, trans):
    transa, transb = trans
    rng = G.rng_for(60 + 4 * (layout == "C") + ["NN", "TN", "NT", "TT"].index(trans))
    for si, (m, n, k) in enumerate(SHAPES):
        col = layout == "C"
        ta, tb = transa == "T", transb == "T"
        ar, ac = (k, m) if ta else (m, k)
        br, bc = (n, k) if tb else (k, n)
        lda = (ar if col else ac) + 1
        ldb = (br if col else bc) + 2
        ldc = (m if col else n) + 3
        A = G.uniform_full(rng, (ac if col else ar) * lda)
        B = G.uniform_full(rng, (bc if col else br) * ldb)
        C = G.uniform_full(rng, (n if col else m) * ldc)
        al_d, be_d = [(1.0, 0.0), (2.5, 1.5), (-0.5, -2.0)][si % 3]
        alpha, beta = Q.scalar(al_d), Q.scalar(be_d)
        got = C.copy()
        api.gemm(layout, transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, got, ldc)
        rows, cols = np.meshgrid(np.arange(m), np.arange(n), indexing="ij")
        rows, cols = rows.ravel(), cols.ravel()
        idx, exp, _ = expected_entries(O, layout, transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc,
                                       rows, cols)
        assert Q.same_bits(got[idx], exp).all(), (layout, trans, m, n, k)
        untouched = np.setdiff1d(np.arange(len(C)), idx)
        assert Q.same_bits(got[untouched], C[untouched]).all()


def test_gemm_vs_reference_fixtures(qlib, O):
    gold = np.load(GOLDEN)
    for tag in ("gemm_simple", "gemm_blocked"):
        m, n, k = (int(v) for v in gold[f"{tag}_meta"])
        A, B, C = gold[f"{tag}_A"], gold[f"{tag}_B"], gold[f"{tag}_C"]
        got = C.copy()
        api.qgemm("R", "N", "N", m, n, k, 2.5, A, k, B, n, 1.5, got, n)
        rows, cols = np.meshgrid(np.arange(m), np.arange(n), indexing="ij")
        alpha, beta = Q.scalar(2.5), Q.scalar(1.5)
        idx, exp, ab = expected_entries(O, "R", "N", "N", m, n, k, alpha, A, k, B, n, beta, C, n,
                                        rows.ravel(), cols.ravel())
        assert Q.same_bits(got[idx], exp).all()
        lim = epilogue_bound(O, alpha, ab, beta, C[idx])
        assert O.bound_violations(got[idx], gold[f"{tag}_out"][idx], lim, float(k + 2)) == 0


def test_gemm_512_full_mantissa(qlib, O, torch_cuda):
    """The soft-float qgemm workload: 512^3 row-major, alpha = 1, beta = 0,
    full 113-bit significands, device pointers; 20000 sampled entries
    checked against the exact oracle and every entry against the reduction
    bound of the reference's own order on a 64-row slice."""
    torch = torch_cuda
    m = n = k = 512
    rng = G.rng_for(0xC0FFEE)
    A, B, C = G.uniform_full(rng, m * k), G.uniform_full(rng, k * n), G.uniform_full(rng, m * n)
    dA, dB, dC = to_dev(torch, A), to_dev(torch, B), to_dev(torch, C)
    alpha, beta = Q.scalar(1.0), Q.scalar(0.0)
    api.gemm_dev("R", "N", "N", m, n, k, alpha, dA, k, dB, n, beta, dC, n)
    torch.cuda.synchronize()
    got = to_host(dC)
    rows = rng.integers(0, m, 20000)
    cols = rng.integers(0, n, 20000)
    idx, exp, _ = expected_entries(O, "R", "N", "N", m, n, k, alpha, A, k, B, n, beta, C, n, rows, cols)
    assert Q.same_bits(got[idx], exp).all()
    ref = O.ref_gemm(0, 64, n, k, alpha, A, k, B, n, beta, C[: 64 * n], n, lib_order=1, nthreads=16)
    rows, cols = np.meshgrid(np.arange(64), np.arange(n), indexing="ij")
    _, _, ab = expected_entries(O, "R", "N", "N", 64, n, k, alpha, A, k, B, n, beta, C, n, rows.ravel(),
                                cols.ravel())
    assert O.bound_violations(got[: 64 * n], ref, ab, float(k + 2)) == 0
