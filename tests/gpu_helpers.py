"""Shared helpers for the GPU parity tests: expected results built from the
oracle, and repetition of a binary128 scalar."""
import numpy as np

from qblas_gb300 import quad as Q


def rep(q1: np.ndarray, n: int) -> np.ndarray:
    return np.repeat(Q.as_quad(q1), n, axis=0)


def qabs(a: np.ndarray) -> np.ndarray:
    a = Q.as_quad(a).copy()
    a[:, 1] &= ~np.uint64(1 << 63)
    return a


def epilogue(O, alpha, R, beta, yold):
    """y = fma(alpha, R, beta * yold), elementwise (the reference epilogue)."""
    n = len(R)
    return O.fma(rep(alpha, n), R, O.mul(rep(beta, n), yold))


def epilogue_bound(O, alpha, absum, beta, yold):
    """|alpha| * sum|a b| + |beta y| per output, the magnitude that the
    reduction bound k * 2^-113 * (...) is taken of (oracle.bound_violations
    applies the factor k * 2^-113)."""
    n = len(absum)
    return O.fma(rep(qabs(alpha), n), absum, qabs(O.mul(rep(beta, n), yold)))


def strided(a: np.ndarray, inc: int) -> np.ndarray:
    """Element i of a strided vector stored with increment inc."""
    return Q.as_quad(a)[::inc]
