"""GPU parity of qgemv against the oracle, through the C ABI.

Tolerance: each y_i must be bit-identical to fma(alpha, R_i, beta*y_i)
where R_i is the correctly rounded exact row sum (exact long accumulator)
and fma/mul are correctly rounded (the reference's epilogue,
level2.hpp:48); against the reference's own FMA-chain outputs the
difference must stay within (n + 2) * u_q * (|alpha| sum|a x| + |beta y|).
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


def op_strides(layout, trans, lda):
    """(m', n', si, sj) of op(A) per the reference's trans handling
    (c_interface.hpp:76-85)."""
    col = layout in "Cc"
    if trans in "TtCc":
        col = not col
    return (1, lda) if col else (lda, 1)


def expected(O, layout, trans, m, n, alpha, A, lda, x, incx, beta, y, incy):
    mm, nn = (n, m) if trans in "TtCc" else (m, n)
    si, sj = op_strides(layout, trans, lda)
    R, _, ab = O.exact_gemv(mm, nn, A, si, sj, x, incx)
    out = y.copy()
    yold = y[::incy][:mm]
    out[::incy][:mm] = epilogue(O, alpha, R, beta, yold)
    return out, ab


def test_gemv_known_answers(qlib):
    # test_quadblas.cpp:328-350: [[1,2,3],[4,5,6],[7,8,9]] @ [1,1,1] = [6,15,24]
    A = Q.from_double(np.arange(1, 10))
    x = Q.from_double(np.ones(3))
    y = Q.from_double(np.zeros(3))
    api.qgemv("R", "N", 3, 3, 1.0, A, 3, x, 1, 0.0, y, 1)
    assert np.array_equal(Q.to_double_approx(y), [6, 15, 24])
    # tests/test_sleef_simd.cpp:87-110: [[1,2],[3,4]] @ [1,1] = [3,7]
    A = Q.from_double([1, 2, 3, 4])
    y = Q.from_double(np.zeros(2))
    api.qgemv("R", "N", 2, 2, 1.0, A, 2, Q.from_double([1, 1]), 1, 0.0, y, 1)
    assert np.array_equal(Q.to_double_approx(y), [3, 7])


CASES = [(1, 1), (3, 7), (100, 100), (129, 257), (37, 1000), (1000, 37), (16, 2048)]
SCALARS = [(1.0, 0.0), (1.5, 0.5), (-2.0, 3.0)]


@pytest.mark.parametrize("layout", ["R", "C"])
@pytest.mark.parametrize("trans", ["N", "T"])
def test_gemv_bit_exact(qlib, O, layout, trans):
    rng = G.rng_for(40 + 2 * (layout == "C") + (trans == "T"))
    for ci, (m, n) in enumerate(CASES):
        for incx, incy in [(1, 1), (2, 3)]:
            al_d, be_d = SCALARS[ci % len(SCALARS)]
            mm, nn = (n, m) if trans == "T" else (m, n)
            col = (layout == "C")
            pad = 3
            lda = (m if col else n) + pad
            A = G.uniform_full(rng, (n if col else m) * lda)
            x = G.uniform_full(rng, nn * incx)
            y = G.uniform_full(rng, mm * incy)
            alpha, beta = Q.scalar(al_d), Q.scalar(be_d)
            got = y.copy()
            api.gemv(layout, trans, m, n, alpha, A, lda, x, incx, beta, got, incy)
            exp, _ = expected(O, layout, trans, m, n, alpha, A, lda, x, incx, beta, y, incy)
            assert Q.same_bits(got, exp).all(), (layout, trans, m, n, incx, incy)
            # reference C interface (double scalars)
            got2 = y.copy()
            api.qgemv(layout, trans, m, n, al_d, A, lda, x, incx, be_d, got2, incy)
            assert Q.same_bits(got2, exp).all()


def test_gemv_vs_reference_order(qlib, O):
    """Within the reduction bound of the reference's own order (library
    order, both layouts) and of the committed reference fixtures."""
    gold = np.load(GOLDEN)
    for tag in ("gemv_row", "gemv_col"):
        cm, m, n, lda = (int(v) for v in gold[f"{tag}_meta"])
        A, x, y = gold[f"{tag}_A"], gold[f"{tag}_x"], gold[f"{tag}_y"]
        alpha, beta = Q.scalar(1.5), Q.scalar(0.5)
        got = y.copy()
        api.qgemv("C" if cm else "R", "N", m, n, 1.5, A, lda, x, 1, 0.5, got, 1)
        exp, ab = expected(O, "C" if cm else "R", "N", m, n, alpha, A, lda, x, 1, beta, y, 1)
        assert Q.same_bits(got, exp).all()
        lim = epilogue_bound(O, alpha, ab, beta, y)
        assert O.bound_violations(got, gold[f"{tag}_out"], lim, float(n + 2)) == 0


def test_gemv_nan_propagation(qlib, O):
    # beta = 0 still multiplies y (level2.hpp:48): NaN in y stays NaN
    A = Q.from_double(np.ones(4))
    x = Q.from_double(np.ones(2))
    y = Q.from_double([np.nan, 1.0])
    api.qgemv("R", "N", 2, 2, 1.0, A, 2, x, 1, 0.0, y, 1)
    assert Q.is_nan(y)[0] and Q.to_double_approx(y)[1] == 2.0


def test_gemv_full_size_row_major(qlib, O, torch_cuda):
    """The qgemv benchmark workload: 8192 x 8192 row-major on the
    wide-exponent distribution, device pointers, checked entry by entry
    against the exact oracle."""
    torch = torch_cuda
    m = n = 8192
    rng = G.rng_for(2)
    A = G.wide_exponent(rng, m * n)
    x = G.wide_exponent(rng, n)
    y = G.wide_exponent(rng, m)
    dA, dx, dy = to_dev(torch, A), to_dev(torch, x), to_dev(torch, y)
    alpha, beta = Q.scalar(1.0), Q.scalar(0.0)
    api.gemv_dev("R", "N", m, n, alpha, dA, n, dx, 1, beta, dy, 1)
    torch.cuda.synchronize()
    got = to_host(dy)
    R, _, _ = O.exact_gemv(m, n, A, n, 1, x, 1, nthreads=16)
    exp = epilogue(O, alpha, R, beta, y)
    assert Q.same_bits(got, exp).all()


def test_gemv_full_size_col_major(qlib, O, torch_cuda):
    torch = torch_cuda
    m, n = 4096, 8192
    rng = G.rng_for(4)
    A = G.wide_exponent(rng, m * n)  # column-major, lda = m
    x = G.wide_exponent(rng, n)
    y = G.wide_exponent(rng, m)
    dA, dx, dy = to_dev(torch, A), to_dev(torch, x), to_dev(torch, y)
    alpha, beta = Q.scalar(0.5), Q.scalar(2.0)
    api.gemv_dev("C", "N", m, n, alpha, dA, m, dx, 1, beta, dy, 1)
    torch.cuda.synchronize()
    got = to_host(dy)
    R, _, _ = O.exact_gemv(m, n, A, 1, m, x, 1, nthreads=16)
    assert Q.same_bits(got, epilogue(O, alpha, R, beta, y)).all()
