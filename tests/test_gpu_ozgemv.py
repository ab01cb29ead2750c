"""GPU parity of the Ozaki-split qgemv (tensor cores, certified rounding),
through the C ABI with quadblas_set_method(2).

Tolerance: none.  Every y_i must be bit-identical to fma(alpha, R_i, beta*y_i)
with R_i the correctly rounded exact row sum (the exact oracle), as for the
soft-float kernels: rows the Ozaki bound cannot certify (NaN / inf, wide
exponent spreads, heavy cancellation) are recomputed exactly, so the
result does not depend on which rows took which path.
"""
import numpy as np
import pytest

from qblas_gb300 import api
from qblas_gb300 import gen as G
from qblas_gb300 import quad as Q
from gpu_helpers import epilogue
from test_gpu_level2 import expected

pytestmark = pytest.mark.gpu

CASES = [(1, 1), (5, 40), (128, 32), (129, 33), (300, 1000), (1000, 300), (2048, 512)]


@pytest.fixture
def ozaki():
    api.set_method(2)
    yield
    api.set_method(0)


def run(O, layout, trans, m, n, A, lda, x, incx, y, incy, al=1.0, be=0.0):
    alpha, beta = Q.scalar(al), Q.scalar(be)
    got = y.copy()
    api.gemv(layout, trans, m, n, alpha, A, lda, x, incx, beta, got, incy)
    exp, _ = expected(O, layout, trans, m, n, alpha, A, lda, x, incx, beta, y, incy)
    return got, exp


@pytest.mark.parametrize("layout", ["R", "C"])
@pytest.mark.parametrize("trans", ["N", "T"])
def test_ozgemv_bit_exact(qlib, O, ozaki, layout, trans):
    rng = G.rng_for(140 + 2 * (layout == "C") + (trans == "T"))
    for ci, (m, n) in enumerate(CASES):
        for incx, incy in [(1, 1), (2, 3)]:
            mm, nn = (n, m) if trans == "T" else (m, n)
            col = layout == "C"
            lda = (m if col else n) + 3
            gen = G.wide_exponent if ci % 2 else G.uniform_full
            A = gen(rng, (n if col else m) * lda)
            x = gen(rng, nn * incx)
            y = G.uniform_full(rng, mm * incy)
            al, be = [(1.0, 0.0), (1.5, 0.5), (-2.0, 3.0)][ci % 3]
            got, exp = run(O, layout, trans, m, n, A, lda, x, incx, y, incy, al, be)
            assert Q.same_bits(got, exp).all(), (layout, trans, m, n, incx, incy)


def test_ozgemv_hard_rows(qlib, O, ozaki):
    """Rows that need the exact pass next to rows that certify."""
    rng = G.rng_for(150)
    m, n = 512, 640
    A = G.uniform_full(rng, m * n).reshape(m, n, 2)
    x = G.uniform_full(rng, n)
    # rows 0-63: cancelling dot products (GenDot-like: pairs cancel to 2^-80)
    for i in range(64):
        a, _ = G.cancelling_dot(G.rng_for(1000 + i), n)
        A[i] = a
    # rows 64-127: exponents spread over +-2000 inside every chunk
    A[64:128] = G.spread_uniform(rng, 64 * n, -2000, 2000).reshape(64, n, 2)
    # row 128 all zero, row 129 negative zeros, row 130 subnormal
    A[128] = 0
    A[129] = 0
    A[129, :, 1] = np.uint64(1 << 63)
    sub = G.uniform_full(rng, n)
    sub[:, 1] &= ~np.uint64(0x7FFF << 48)
    A[130] = sub
    # row 131 holds +inf, row 132 NaN, row 133 +inf and -inf
    A[131, 5] = [0, 0x7FFF << 48]
    A[132, 7] = [1, 0x7FFF << 48]
    A[133, 1] = [0, 0x7FFF << 48]
    A[133, 2] = [0, (0xFFFF << 48)]
    A = A.reshape(-1, 2)
    y = G.uniform_full(rng, m)
    got, exp = run(O, "R", "N", m, n, A, n, x, 1, y, 1, 1.0, 0.5)
    assert Q.same_bits(got, exp).all(), np.argwhere(~Q.same_bits(got, exp))[:5]


def test_ozgemv_special_x(qlib, O, ozaki):
    rng = G.rng_for(151)
    m, n = 300, 200
    A = G.uniform_full(rng, m * n)
    A[:n][::7] = 0  # some zeros in row 0: 0 * inf = NaN there
    for pos, hi in [(17, 0x7FFF << 48), (40, (1 << 63) | (0x7FFF << 48)), (199, (0x7FFF << 48) | 1)]:
        x = G.uniform_full(rng, n)
        x[pos] = [0, hi]
        got, exp = run(O, "R", "N", m, n, A, n, x, 1, G.uniform_full(rng, m), 1)
        assert Q.same_bits(got, exp).all(), pos


def test_ozgemv_zero_x_and_empty(qlib, O, ozaki):
    rng = G.rng_for(152)
    m, n = 200, 100
    A = G.wide_exponent(rng, m * n)
    x = np.zeros((n, 2), dtype=np.uint64)
    got, exp = run(O, "R", "N", m, n, A, n, x, 1, G.uniform_full(rng, m), 1, 2.0, 1.0)
    assert Q.same_bits(got, exp).all()
    y = G.uniform_full(rng, 4)
    got = y.copy()
    api.gemv("R", "N", 4, 0, Q.scalar(1.0), np.zeros((1, 2), np.uint64), 1, np.zeros((1, 2), np.uint64), 1,
             Q.scalar(0.0), got, 1)
    assert Q.same_bits(got, y).all()  # n == 0 leaves y untouched, as the reference


@pytest.mark.parametrize("layout", ["R", "C"])
def test_methods_agree(qlib, O, layout):
    """Auto, soft-float and Ozaki give the same bits."""
    rng = G.rng_for(153 + (layout == "C"))
    m, n = 4096, 1100
    A = G.wide_exponent(rng, m * n)
    x = G.wide_exponent(rng, n)
    y = G.uniform_full(rng, m)
    outs = []
    try:
        for method in (0, 1, 2):
            api.set_method(method)
            got = y.copy()
            api.gemv(layout, "N", m, n, Q.scalar(1.0), A, n if layout == "R" else m, x, 1, Q.scalar(0.25), got, 1)
            outs.append(got)
    finally:
        api.set_method(0)
    assert Q.same_bits(outs[0], outs[1]).all() and Q.same_bits(outs[2], outs[1]).all()
    rows = np.arange(0, m, 97)
    lda = n if layout == "R" else m
    si, sj = (lda, 1) if layout == "R" else (1, lda)
    R, _, _ = O.exact_gemv(m, n, A, si, sj, x, 1)
    exp = epilogue(O, Q.scalar(1.0), R, Q.scalar(0.25), y)
    assert Q.same_bits(outs[2][rows], exp[rows]).all()


@pytest.mark.parametrize("kind", ["wide", "uniform"])
def test_certified_rows(qlib, O, ozaki, kind):
    """Almost every row certifies (the exact pass is for hard rows only)."""
    rng = G.rng_for(155 + (kind == "uniform"))
    m, n = 2048, 4096
    gen = G.wide_exponent if kind == "wide" else G.uniform_full
    A, x = gen(rng, m * n), gen(rng, n)
    api.debug_count_exact_rows(True)
    try:
        got = np.zeros((m, 2), dtype=np.uint64)
        api.gemv("R", "N", m, n, Q.scalar(1.0), A, n, x, 1, Q.scalar(0.0), got, 1)
        exact_rows = api.debug_exact_rows()
    finally:
        api.debug_count_exact_rows(False)
    print(f"\n{kind}: {exact_rows} of {m} rows recomputed exactly")
    assert 0 <= exact_rows <= m // 100
    rows = np.arange(0, m, 61)
    R, _, _ = O.exact_gemv(m, n, A, n, 1, x, 1)
    assert Q.same_bits(got[rows], R[rows]).all()


@pytest.mark.parametrize("cond", [1e10, 1e20, 1e30, 1e40])
def test_ozgemv_gendot_rows(qlib, O, ozaki, cond):
    """A row of prescribed condition (GenDot) among random rows: the Ozaki bound
    cannot certify heavy cancellation, so that row goes to the exact pass."""
    n, m = 8192, 300
    X, Y = O.gendot_batch(n, np.array([cond]), np.array([77], dtype=np.uint64))
    rng = G.rng_for(160)
    A = G.uniform_full(rng, m * n).reshape(m, n, 2)
    A[5] = X.reshape(n, 2)
    A = A.reshape(-1, 2)
    x = np.ascontiguousarray(Y.reshape(n, 2))
    api.debug_count_exact_rows(True)
    try:
        got, exp = run(O, "R", "N", m, n, A, n, x, 1, G.uniform_full(rng, m), 1, 1.0, 0.0)
        listed = api.debug_exact_rows()
    finally:
        api.debug_count_exact_rows(False)
    assert Q.same_bits(got, exp).all()
    if cond >= 1e30:
        assert listed >= 1


def test_ozgemv_no_memory(qlib, O, ozaki, torch_cuda):
    """An injected allocation failure: status NO_MEMORY, y untouched, then a
    normal call."""
    import ctypes

    from conftest import to_dev, to_host
    torch = torch_cuda
    rng = G.rng_for(161)
    m, n = 256, 640
    A, x, y0 = G.uniform_full(rng, m * n), G.uniform_full(rng, n), G.uniform_full(rng, m)
    dA, dx, dy = to_dev(torch, A), to_dev(torch, x), to_dev(torch, y0)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    one, zero = Q.scalar(1.0), Q.scalar(0.0)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    D = lambda t: ctypes.c_void_p(t.data_ptr())
    qlib.quadblas_debug_fail_allocations(1)
    try:
        rc = qlib.quadblas_qgemv_dev(b"R", b"N", m, n, P(one), D(dA), n, D(dx), 1, P(zero), D(dy), 1, s)
    finally:
        qlib.quadblas_debug_fail_allocations(0)
    assert rc == 3
    torch.cuda.synchronize()
    assert Q.same_bits(to_host(dy), y0).all()
    assert qlib.quadblas_qgemv_dev(b"R", b"N", m, n, P(one), D(dA), n, D(dx), 1, P(zero), D(dy), 1, s) == 0
    torch.cuda.synchronize()
    R, _, _ = O.exact_gemv(m, n, A, n, 1, x, 1)
    assert Q.same_bits(to_host(dy), R).all()
