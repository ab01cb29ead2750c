"""The exact fallback and the rounding certificate (exact.cuh, compiled for
the host) against the oracle's exact long accumulator.

* The Kulisch dot is bit-exact with the correctly rounded exact sum on every
  input class: uniform, full exponent range, subnormal, cancelling, GenDot up
  to condition 1e40, NaN / infinity / zero operands, empty.
* The certificate is sound: whenever the wide-accumulator result is
  certified it equals the correctly rounded exact sum (any chunking); and it
  is not vacuous: well-conditioned sums are certified, GenDot sums at
  condition 1e40 are not."""
import ctypes

import numpy as np
import pytest

import quadvec as V
from qblas_gb300 import gen as G
from qblas_gb300 import quad as Q

c64 = ctypes.c_int64


def P(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def kulisch(sq, x, y):
    x, y = np.ascontiguousarray(x), np.ascontiguousarray(y)
    out = Q.empty(1)
    sq.sq_kulisch_dot(c64(len(x)), P(x), c64(1), P(y), c64(1), P(out))
    return out


def certified(sq, x, y, nsplit):
    x, y = np.ascontiguousarray(x), np.ascontiguousarray(y)
    out, ok = Q.empty(1), np.zeros(1, np.int32)
    sq.sq_wacc_dot_certified(c64(len(x)), P(x), P(y), c64(nsplit), P(out), P(ok))
    return out, bool(ok[0])


def cases(O):
    rng = G.rng_for(31)
    yield "uniform", G.uniform_full(rng, 500), G.uniform_full(rng, 500)
    yield "wide", G.wide_exponent(rng, 700, -60, 60), G.wide_exponent(rng, 700, -60, 60)
    yield "full range", V.finite(rng, 300, -8000, 8000), V.finite(rng, 300, -8000, 8000)
    yield "huge", V.finite(rng, 50, 16000, 16383), V.finite(rng, 50, -16000, -15000)
    yield "subnormal", V.subnormal(rng, 200), V.finite(rng, 200, -10, 10)
    yield "tiny products", V.subnormal(rng, 100), V.subnormal(rng, 100)
    x, y = G.cancelling_dot(rng, 1000, -200, 200)
    yield "cancelling", x, y
    xn = x.copy()
    xn[:, 1] ^= np.uint64(1 << 63)
    yield "exact zero", np.concatenate([x, xn]), np.concatenate([y, y])
    for cond in (1e10, 1e20, 1e30, 1e40):
        x, y = O.gendot(2048, cond, 17)
        yield f"gendot {cond:.0e}", x, y
    yield "empty", Q.empty(0), Q.empty(0)


def test_kulisch_dot_is_exact(O, sq):
    for name, x, y in cases(O):
        R, _, _ = O.exact_dot(x, y)
        assert Q.same_bits(kulisch(sq, x, y), R).all(), name


def test_kulisch_dot_specials(O, sq):
    rng = G.rng_for(32)
    sp = V.specials()
    for t in range(60):
        x, y = G.uniform_full(rng, 16), G.uniform_full(rng, 16)
        k = int(rng.integers(1, 4))
        idx = rng.integers(0, 16, k)
        x[idx] = sp[rng.integers(0, len(sp), k)]
        R, _, _ = O.exact_dot(x, y)
        assert Q.same_bits(kulisch(sq, x, y), R).all(), t


@pytest.mark.parametrize("nsplit", [1, 7, 256])
def test_certificate_is_sound(O, sq, nsplit):
    n_cert = 0
    for name, x, y in cases(O):
        got, ok = certified(sq, x, y, nsplit)
        if ok:
            n_cert += 1
            R, _, _ = O.exact_dot(x, y)
            assert Q.same_bits(got, R).all(), name
    assert n_cert >= 8


def test_certificate_is_not_vacuous(O, sq):
    rng = G.rng_for(33)
    for _ in range(20):
        x, y = G.wide_exponent(rng, 1000), G.wide_exponent(rng, 1000)
        assert certified(sq, x, y, 16)[1]
    x, y = O.gendot(4096, 1e40, 5)
    assert not certified(sq, x, y, 1)[1]
    # an exact tie (1 + 2^-113) is rounded to even but cannot be certified
    x = np.concatenate([Q.scalar(1.0), Q.scalar(2.0 ** -113)])
    y = np.concatenate([Q.scalar(1.0), Q.scalar(1.0)])
    got, ok = certified(sq, x, y, 1)
    assert Q.same_bits(got, Q.scalar(1.0)).all()


def trunc_certified(sq, x, y, nsplit):
    x, y = np.ascontiguousarray(x), np.ascontiguousarray(y)
    out, ok = Q.empty(1), np.zeros(1, np.int32)
    sq.sq_wacc_dot_trunc_certified(c64(len(x)), P(x), P(y), c64(nsplit), P(out), P(ok))
    return out, bool(ok[0])


def test_truncated_product_bound(sq):
    """The qdot kernel's products (limbs 2..7 without the partial products of
    limbs 0 and 1) are at most 4 units of limb 2 below the exact top bits."""
    rng = G.rng_for(34)
    x = np.concatenate([G.uniform_full(rng, 300), V.subnormal(rng, 50)])
    y = np.concatenate([G.uniform_full(rng, 300), V.finite(rng, 50, -10, 10)])
    x[:20, 0] = np.uint64(0xFFFFFFFFFFFFFFFF)  # all-ones low words: the largest dropped carries
    y[:20, 0] = np.uint64(0xFFFFFFFFFFFFFFFF)
    out = np.zeros((len(x), 6), dtype=np.uint32)
    sq.sq_mul_top192(c64(len(x)), P(x), P(y), P(out))

    def sig(w):  # significand shifted to bit 127, as the device unpacks it
        lo, hi = int(w[0]), int(w[1])
        be = (hi >> 48) & 0x7FFF
        m = ((hi & ((1 << 48) - 1)) << 64) | lo
        if be:
            m |= 1 << 112
        return m << (127 - (m.bit_length() - 1)) if m else 0

    for i in range(len(x)):
        exact = (sig(x[i]) * sig(y[i])) >> 64
        got = sum(int(out[i, k]) << (32 * k) for k in range(6))
        assert 0 <= exact - got < 4, i


@pytest.mark.parametrize("nsplit", [1, 256])
def test_truncated_certificate_is_sound(O, sq, nsplit):
    """Certified sums of truncated products equal the correctly rounded exact sum."""
    n_cert = 0
    for name, x, y in cases(O):
        got, ok = trunc_certified(sq, x, y, nsplit)
        if ok:
            n_cert += 1
            R, _, _ = O.exact_dot(x, y)
            assert Q.same_bits(got, R).all(), name
    assert n_cert >= 6
    rng = G.rng_for(35)
    x, y = G.cancelling_dot(rng, 4096)  # the benchmark's data kind certifies
    assert trunc_certified(sq, x, y, nsplit)[1]
