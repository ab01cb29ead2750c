"""GPU parity of qdot / qnrm2 / qaxpy against the oracle, through the C ABI.

Tolerances (binary128, u_q = 2^-113):
  * dot / nrm2: the result must equal the correctly rounded exact sum
    (bit-exact against the exact long accumulator; 0.5 ulp), and lie within
    n * u_q * sum|x_i y_i| of the reference's own FMA-chain result.
  * axpy: bit-exact with fma(alpha, x_i, y_i), i.e. with the reference.
"""
import ctypes
import os

import numpy as np
import pytest

import quadvec as V
from conftest import to_dev, to_host
from gpu_helpers import rep
from qblas_gb300 import api
from qblas_gb300 import gen as G
from qblas_gb300 import quad as Q

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_outputs.npz")


def P(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def test_dot_known_answers(qlib, O):
    # test_quadblas.cpp:205-224: dot(1..10, 1) = 55; :715-739: 1e20 + 1 - 1e20 = 1;
    # tests/test_sleef_simd.cpp:57,61: dot(1..5, 1) = 15
    x = Q.from_double(np.arange(1, 11))
    one = Q.from_double(np.ones(10))
    assert Q.same_bits(api.dot(x, one), Q.scalar(55.0)).all()
    assert api.qdot(10, x, 1, one, 1) == 55.0
    assert api.qdot(5, x, 1, one, 1) == 15.0
    v, w = Q.from_double([1e20, 1.0, -1e20]), Q.from_double([1.0, 1.0, 1.0])
    assert api.qdot(3, v, 1, w, 1) == 1.0
    assert api.qdot(0, x, 1, one, 1) == 0.0


@pytest.mark.parametrize("kind", ["uniform", "cancel", "wide", "mixed", "tiny", "sparse"])
def test_dot_correctly_rounded(qlib, O, kind):
    rng = G.rng_for(100 + ["uniform", "cancel", "wide", "mixed", "tiny", "sparse"].index(kind))
    for n in (1, 2, 31, 32, 33, 257, 1000, 4099, 65537, 300001):
        if kind == "uniform":
            x, y = G.uniform_full(rng, n), G.uniform_full(rng, n)
        elif kind == "cancel":
            x, y = G.cancelling_dot(rng, max(n, 4))
        elif kind == "wide":
            x, y = G.wide_exponent(rng, n, -16000, 16000), G.wide_exponent(rng, n, -300, 300)
        elif kind == "mixed":
            x, y = V.mixed(rng, n), V.mixed(rng, n)
        elif kind == "tiny":
            x, y = V.finite(rng, n, -16382, -16300), V.finite(rng, n, -100, 0)
        else:
            x, y = V.finite(rng, n, -5, 5, sparse=True), V.finite(rng, n, -5, 5, sparse=True)
        n = len(x)
        got = api.dot(x, y)
        R, r, ab = O.exact_dot(x, y)
        assert Q.same_bits(got, R).all(), (kind, n, O.ulp_err(got, R, r))
        if kind in ("uniform", "cancel"):
            ref = O.ref_dot(x, y, nthreads=8)
            assert O.bound_violations(got, ref, ab, float(n)) == 0


def test_dot_strided(qlib, O):
    rng = G.rng_for(7)
    for n, incx, incy in [(1000, 3, 2), (77, 2, 5), (100001, 1, 4)]:
        x, y = G.uniform_full(rng, n * incx), G.uniform_full(rng, n * incy)
        got = api.dot(x, y, n, incx, incy)
        R, _, _ = O.exact_dot(x, y, n, incx, incy)
        assert Q.same_bits(got, R).all()


def test_dot_special_values(qlib, O):
    one = Q.scalar(1.0)
    nan = np.array([[0, 0x7FFF800000000000]], dtype=np.uint64)
    inf = np.array([[0, 0x7FFF000000000000]], dtype=np.uint64)
    ninf = np.array([[0, 0xFFFF000000000000]], dtype=np.uint64)
    big = np.array([[(1 << 64) - 1, 0x7FFEFFFFFFFFFFFF]], dtype=np.uint64)
    zero = Q.scalar(0.0)
    cases = [
        (np.concatenate([one, nan]), np.concatenate([one, one])),         # NaN
        (np.concatenate([one, inf]), np.concatenate([one, one])),         # +inf
        (np.concatenate([inf, ninf]), np.concatenate([one, one])),        # inf - inf
        (np.concatenate([inf, one]), np.concatenate([zero, one])),        # inf * 0
        (np.concatenate([big, big]), np.concatenate([big, big])),         # overflow
        (np.concatenate([big, big]), np.concatenate([one, one])),         # max + max
    ]
    for x, y in cases:
        got = api.dot(x, y)
        R, _, _ = O.exact_dot(x, y)
        assert Q.same_bits(got, R).all(), (x, y, got, R)


def test_dot_device_pointers_full_size(qlib, O, torch_cuda):
    """qdot n = 2^26 on the wide-exponent cancelling distribution (the qdot
    benchmark workload), through the device-pointer entry point, against the
    exact oracle at full size."""
    torch = torch_cuda
    n = 1 << 26
    x, y = G.cancelling_dot(G.rng_for(1), n)
    dx, dy = to_dev(torch, x), to_dev(torch, y)
    dres = torch.zeros((1, 2), dtype=torch.int64, device="cuda")
    api.dot_dev(n, dx, 1, dy, 1, dres)
    torch.cuda.synchronize()
    got = to_host(dres)
    R, r, _ = O.exact_dot(x, y)
    assert Q.same_bits(got, R).all(), O.ulp_err(got, R, r)
    # reproducible run to run
    api.dot_dev(n, dx, 1, dy, 1, dres)
    assert Q.same_bits(to_host(dres), got).all()


def test_dot_matches_reference_fixtures(qlib, O):
    gold = np.load(GOLDEN)
    for name in ("dot_small", "dot_par", "dot_strided", "dot_strided_small"):
        n, incx, incy, _ = (int(v) for v in gold[f"{name}_meta"])
        x, y = gold[f"{name}_x"], gold[f"{name}_y"]
        got = api.dot(x, y, n, incx, incy)
        R, _, ab = O.exact_dot(x, y, n, incx, incy)
        assert Q.same_bits(got, R).all()
        assert O.bound_violations(got, gold[f"{name}_out"], ab, float(n)) == 0


def test_nrm2(qlib, O):
    # test_quadblas.cpp:290-312: norm of 1..1000 against sqrt(n(n+1)(2n+1)/6)
    x = Q.from_double(np.arange(1, 1001))
    got = api.nrm2(x)
    R, _, _ = O.exact_dot(x, x)
    assert Q.same_bits(got, O.sqrt(R)).all()
    assert abs(api.qnrm2(1000, x, 1) - np.sqrt(1000 * 1001 * 2001 / 6)) < 1e-12 * np.sqrt(1000)
    # tests/test_sleef_simd.cpp:81-84: norm of 1..5 = sqrt(55)
    assert api.qnrm2(5, x, 1) == float(np.sqrt(55.0))
    rng = G.rng_for(3)
    y = G.uniform_full(rng, 12345)
    R, _, _ = O.exact_dot(y, y)
    assert Q.same_bits(api.nrm2(y), O.sqrt(R)).all()


def test_axpy_bit_exact(qlib, O):
    rng = np.random.default_rng(5)
    for n, incx, incy in [(1, 1, 1), (5000, 1, 1), (777, 2, 3), (100003, 1, 1)]:
        x, y = V.mixed(rng, n * incx), V.mixed(rng, n * incy)
        alpha = V.finite(rng, 1, -10, 10)
        yy = y.copy()
        api.axpy(alpha, x, yy, n, incx, incy)
        exp = y.copy()
        exp[::incy][:n] = O.fma(rep(alpha, n), x[::incx][:n], y[::incy][:n])
        assert Q.same_bits(yy, exp).all()
    # reference C interface with a double alpha, against the reference's own output
    gold = np.load(GOLDEN)
    yy = gold["axpy_y"].copy()
    api.qaxpy(1000, 2.5, gold["axpy_x"], 1, yy, 1)
    assert Q.same_bits(yy, gold["axpy_out"]).all()


def test_axpy_device_pointers(qlib, O, torch_cuda):
    torch = torch_cuda
    rng = np.random.default_rng(8)
    n = 1 << 20
    x, y = V.mixed(rng, n), V.mixed(rng, n)
    alpha = Q.scalar(-1.25)
    dx, dy = to_dev(torch, x), to_dev(torch, y)
    api.axpy_dev(n, alpha, dx, 1, dy, 1)
    torch.cuda.synchronize()
    assert Q.same_bits(to_host(dy), O.fma(rep(alpha, n), x, y)).all()
