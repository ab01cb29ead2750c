"""The device soft-float core (softquad.cuh) and wide accumulator
(wacc.cuh), compiled as host C++, against the oracle: elementwise
operations bit-exact with the correctly rounded host binary128 library,
and accumulated dot products equal to the correctly rounded exact sum."""
import ctypes

import numpy as np

import quadvec as V
from qblas_gb300 import gen as G
from qblas_gb300 import quad as Q


def _run(sq, name, *args):
    n = len(args[0])
    out = np.zeros((n, 2), dtype=np.uint64)
    getattr(sq, name)(ctypes.c_int64(n), *[a.ctypes.data_as(ctypes.c_void_p) for a in args],
                      out.ctypes.data_as(ctypes.c_void_p))
    return out


def test_elementwise_bit_exact(O, sq):
    rng = np.random.default_rng(2024)
    N = 60000
    a, b, c = V.mixed(rng, N), V.mixed(rng, N), V.mixed(rng, N)
    assert Q.same_bits(O.mul(a, b), _run(sq, "sq_mul_n", a, b)).all()
    assert Q.same_bits(O.add(a, b), _run(sq, "sq_add_n", a, b)).all()
    assert Q.same_bits(O.sub(a, b), _run(sq, "sq_sub_n", a, b)).all()
    assert Q.same_bits(O.fma(a, b, c), _run(sq, "sq_fma_n", a, b, c)).all()
    assert Q.same_bits(O.sqrt(a), _run(sq, "sq_sqrt_n", a)).all()


def test_fma_cancellation_and_ties(O, sq):
    rng = np.random.default_rng(7)
    N = 40000
    a, b = V.finite(rng, N, -100, 100), V.finite(rng, N, -100, 100)
    c = O.mul(a, b)
    c[:, 1] ^= np.uint64(1 << 63)
    c[:, 0] ^= rng.integers(0, 1 << 20, size=N, dtype=np.uint64)
    assert Q.same_bits(O.fma(a, b, c), _run(sq, "sq_fma_n", a, b, c)).all()
    a, b, c = (V.finite(rng, N, -4, 4, sparse=True) for _ in range(3))
    assert Q.same_bits(O.fma(a, b, c), _run(sq, "sq_fma_n", a, b, c)).all()
    assert Q.same_bits(O.add(a, c), _run(sq, "sq_add_n", a, c)).all()


def test_conversions(O, sq):
    rng = np.random.default_rng(3)
    d = rng.standard_normal(20000) * np.exp(rng.uniform(-700, 700, 20000))
    d[:8] = [0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -1e-310, 1.7976931348623157e308]
    ref = O.from_double(d)
    assert Q.same_bits(ref, _run(sq, "sq_from_double_n", d.view(np.uint64))).all()
    assert Q.same_bits(ref, Q.from_double(d)).all()
    x = V.mixed(rng, 20000)
    out = np.zeros(len(x), dtype=np.uint64)
    sq.sq_to_double_n(ctypes.c_int64(len(x)), x.ctypes.data_as(ctypes.c_void_p),
                      out.ctypes.data_as(ctypes.c_void_p))
    refd = O.to_double(x)
    got = out.view(np.float64)
    assert ((refd.view(np.uint64) == out) | (np.isnan(refd) & np.isnan(got))).all()


def test_wide_accumulator_correctly_rounded(O, sq):
    rng = G.rng_for(3)
    for t in range(120):
        n = int(rng.integers(1, 2500))
        kind = t % 6
        if kind == 0:
            x, y = G.uniform_full(rng, n), G.uniform_full(rng, n)
        elif kind == 1:
            x, y = G.cancelling_dot(rng, max(n, 4))
        elif kind == 2:
            x, y = G.wide_exponent(rng, n, -16000, 16000), G.wide_exponent(rng, n, -300, 300)
        elif kind == 3:
            x, y = V.mixed(rng, n), V.mixed(rng, n)
        elif kind == 4:
            x, y = V.finite(rng, n, -16382, -16300), V.finite(rng, n, -100, 0)
        else:
            x, y = V.finite(rng, n, -5, 5, sparse=True), V.finite(rng, n, -5, 5, sparse=True)
        R, r, _ = O.exact_dot(x, y)
        for nsplit in (1, 9, 64):
            g = np.zeros((1, 2), dtype=np.uint64)
            sq.sq_wacc_dot(ctypes.c_int64(len(x)), x.ctypes.data_as(ctypes.c_void_p), ctypes.c_int64(1),
                           y.ctypes.data_as(ctypes.c_void_p), ctypes.c_int64(1), ctypes.c_int64(nsplit),
                           g.ctypes.data_as(ctypes.c_void_p))
            assert Q.same_bits(g, R).all(), (t, kind, nsplit, O.ulp_err(g, R, r))


def test_epilogue_fast_paths(O, sq):
    """y = fma(alpha, sum, beta * y) (the reference epilogue, level2.hpp:48,
    level3.hpp:107) with its shortcuts for beta = +-0 (beta * y a signed zero
    when y is finite; alpha = 1 or any alpha) against the oracle's fma and mul:
    signed zeros, infinities, NaNs, subnormals and underflowing products."""
    rng = np.random.default_rng(31)
    N = 30000
    vals = V.mixed(rng, N)
    special = Q.from_double([0.0, -0.0, np.inf, -np.inf, np.nan, 1.0, -1.0, 2.0 ** -1070, -(2.0 ** -1070)])
    tiny = V.finite(rng, 64, -16400, -16300)
    pool = np.concatenate([vals, special, tiny])
    pick = lambda: pool[rng.integers(0, len(pool), N)]  # noqa: E731
    zeros = Q.from_double(rng.choice([0.0, -0.0], N))
    ones = Q.from_double(np.ones(N))
    for alpha, beta in [(ones, zeros), (pick(), zeros), (ones, pick()), (pick(), pick())]:
        s_, y = pick(), pick()
        s_[:50] = Q.from_double(rng.choice([0.0, -0.0], 50))
        got = np.zeros((N, 2), dtype=np.uint64)
        P = lambda a: np.ascontiguousarray(a).ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        a_, b_ = np.ascontiguousarray(alpha), np.ascontiguousarray(beta)
        sq.sq_epilogue_n(ctypes.c_int64(N), P(a_), P(s_), P(b_), P(y), got.ctypes.data_as(ctypes.c_void_p))
        ref = O.fma(a_, s_, O.mul(b_, y))
        nan_ref = ((ref[:, 1] >> np.uint64(48)) & np.uint64(0x7FFF) == 0x7FFF) & \
                  (((ref[:, 1] & np.uint64((1 << 48) - 1)) | ref[:, 0]) != 0)
        nan_got = ((got[:, 1] >> np.uint64(48)) & np.uint64(0x7FFF) == 0x7FFF) & \
                  (((got[:, 1] & np.uint64((1 << 48) - 1)) | got[:, 0]) != 0)
        assert (nan_ref == nan_got).all()
        assert Q.same_bits(got[~nan_ref], ref[~nan_ref]).all()
