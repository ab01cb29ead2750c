"""ORACLE — test infrastructure only.

ctypes front end of the CPU restatement (``_build/liboracle.so``, built from
``oracle.cpp``) and of the reference itself compiled through the SLEEF shim
(``_ref/libqref.so``, built only where the reference tree exists).  Only
tests, ``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py``
import this module; the product never does.

All binary128 arrays are ``(n, 2)`` uint64 (see ``qblas_gb300/quad.py``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None
c_i64 = ctypes.c_int64
c_vp = ctypes.c_void_p


# The reference checkout whose headers oracle/_ref is compiled from: the
# directory in QBLAS_REFERENCE_DIR, else the read-only mount the reference is
# checked out at on the build machine.  Where neither exists, _ref is skipped.
REFERENCE_DIR = os.environ.get("QBLAS_REFERENCE_DIR", "/root/reference")
# QBLAS_SANITIZE=1: the AddressSanitizer + UndefinedBehaviorSanitizer build
SANITIZE = os.environ.get("QBLAS_SANITIZE", "") not in ("", "0")
BUILD_DIR = os.path.join(HERE, "_build_san" if SANITIZE else "_build")


def build(quiet: bool = True) -> None:
    """Compile the oracle (and oracle/_ref where the reference tree exists)."""
    ref = REFERENCE_DIR if os.path.isfile(os.path.join(REFERENCE_DIR, "include", "quadblas", "quadblas.hpp")) else ""
    san = ["SAN=1"] if SANITIZE else []
    out = subprocess.run(["make", "-C", HERE, f"REF={ref}"] + san, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(BUILD_DIR, "liboracle.so")
        if not os.path.exists(path):
            build()
        _LIB = ctypes.CDLL(path)
        _LIB.oq_count_bound_violations.restype = c_i64
    return _LIB


def ref_lib():
    """The reference compiled from its own headers, or None where absent."""
    global _REF
    if _REF is None:
        path = os.path.join(HERE, "_ref", "libqref.so")
        if not os.path.exists(path):
            return None
        _REF = ctypes.CDLL(path)
        for f in ("qref_c_qdot", "qref_c_qnrm2"):
            getattr(_REF, f).restype = ctypes.c_double
            getattr(_REF, f).argtypes = None
    return _REF


def P(a: np.ndarray):
    return a.ctypes.data_as(c_vp)


def q(a) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.uint64)
    assert a.ndim == 2 and a.shape[1] == 2
    return a


def qs(n):
    return np.zeros((int(n), 2), dtype=np.uint64)


# ---- elementwise ---------------------------------------------------------
def fma(a, b, c):
    a, b, c = q(a), q(b), q(c)
    out = qs(len(a))
    lib().oq_fma_n(c_i64(len(a)), P(a), P(b), P(c), P(out))
    return out


def _binop(name, a, b):
    a, b = q(a), q(b)
    out = qs(len(a))
    getattr(lib(), name)(c_i64(len(a)), P(a), P(b), P(out))
    return out


def mul(a, b):
    return _binop("oq_mul_n", a, b)


def add(a, b):
    return _binop("oq_add_n", a, b)


def sub(a, b):
    return _binop("oq_sub_n", a, b)


def sqrt(a):
    a = q(a)
    out = qs(len(a))
    lib().oq_sqrt_n(c_i64(len(a)), P(a), P(out))
    return out


def from_double(d):
    d = np.ascontiguousarray(d, dtype=np.float64).ravel()
    out = qs(d.size)
    lib().oq_from_double_n(c_i64(d.size), P(d), P(out))
    return out


def to_double(a):
    a = q(a)
    out = np.zeros(len(a), dtype=np.float64)
    lib().oq_to_double_n(c_i64(len(a)), P(a), P(out))
    return out


# ---- reference-order restatement ----------------------------------------
def ref_dot(x, y, n=None, incx=1, incy=1, nthreads=1):
    x, y = q(x), q(y)
    if n is None:
        n = len(x) // incx
    out = qs(1)
    lib().oq_ref_dot(c_i64(n), P(x), c_i64(incx), P(y), c_i64(incy), ctypes.c_int(nthreads), P(out))
    return out


def ref_axpy(alpha, x, y, n=None, incx=1, incy=1, nthreads=1):
    x, y, alpha = q(x), q(y).copy(), q(alpha)
    if n is None:
        n = len(x) // incx
    lib().oq_ref_axpy(c_i64(n), P(alpha), P(x), c_i64(incx), P(y), c_i64(incy), ctypes.c_int(nthreads))
    return y


def ref_gemv(col_major, m, n, alpha, A, lda, x, incx, beta, y, incy, lib_order=0, nthreads=1):
    A, x, alpha, beta = q(A), q(x), q(alpha), q(beta)
    y = q(y).copy()
    lib().oq_ref_gemv(ctypes.c_int(int(col_major)), c_i64(m), c_i64(n), P(alpha), P(A), c_i64(lda),
                      P(x), c_i64(incx), P(beta), P(y), c_i64(incy), ctypes.c_int(lib_order),
                      ctypes.c_int(nthreads))
    return y


def ref_gemm(col_major, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, lib_order=0, nthreads=1):
    A, B, alpha, beta = q(A), q(B), q(alpha), q(beta)
    C = q(C).copy()
    lib().oq_ref_gemm(ctypes.c_int(int(col_major)), c_i64(m), c_i64(n), c_i64(k), P(alpha), P(A),
                      c_i64(lda), P(B), c_i64(ldb), P(beta), P(C), c_i64(ldc), ctypes.c_int(lib_order),
                      ctypes.c_int(nthreads))
    return C


# ---- exact oracle --------------------------------------------------------
def exact_dot(x, y, n=None, incx=1, incy=1):
    """(R, r, absum): R = correctly rounded exact sum, r = round(S - R)."""
    x, y = q(x), q(y)
    if n is None:
        n = len(x) // incx
    R, r, ab = qs(1), qs(1), qs(1)
    lib().oq_exact_dot(c_i64(n), P(x), c_i64(incx), P(y), c_i64(incy), P(R), P(r), P(ab))
    return R, r, ab


def exact_gemv(m, n, A, si, sj, x, incx=1, nthreads=8):
    """Exact rows of op(A) x, op(A)(i, j) = A[i*si + j*sj]."""
    A, x = q(A), q(x)
    R, r, ab = qs(m), qs(m), qs(m)
    lib().oq_exact_gemv(c_i64(m), c_i64(n), P(A), c_i64(si), c_i64(sj), P(x), c_i64(incx), P(R), P(r),
                        P(ab), ctypes.c_int(nthreads))
    return R, r, ab


def exact_gemm(k, A, sai, sal, B, sbl, sbj, rows, cols, nthreads=8):
    """Exact entries (rows[t], cols[t]) of op(A) op(B)."""
    A, B = q(A), q(B)
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    cols = np.ascontiguousarray(cols, dtype=np.int64)
    cnt = rows.size
    R, r, ab = qs(cnt), qs(cnt), qs(cnt)
    lib().oq_exact_gemm(c_i64(k), P(A), c_i64(sai), c_i64(sal), P(B), c_i64(sbl), c_i64(sbj), c_i64(cnt),
                        P(rows), P(cols), P(R), P(r), P(ab), ctypes.c_int(nthreads))
    return R, r, ab


def gendot(n, cond, seed):
    """x, y of length n whose dot product has condition number about `cond`
    (Ogita-Rump-Oishi GenDot, restated for binary128)."""
    x, y = qs(n), qs(n)
    lib().oq_gendot(c_i64(n), ctypes.c_double(cond), ctypes.c_uint64(seed), P(x), P(y))
    return x, y


def gendot_batch(n, conds, seeds, nthreads=None):
    """len(conds) GenDot pairs of length n as (count*n, 2) arrays X, Y: pair p
    occupies rows p*n .. p*n+n-1, with condition about conds[p]."""
    conds = np.ascontiguousarray(conds, dtype=np.float64)
    seeds = np.ascontiguousarray(seeds, dtype=np.uint64)
    cnt = conds.size
    X, Y = qs(cnt * n), qs(cnt * n)
    nt = nthreads or os.cpu_count() or 1
    lib().oq_gendot_batch(c_i64(cnt), c_i64(n), P(conds), P(seeds), P(X), P(Y), ctypes.c_int(nt))
    return X, Y


def dot_condition(x, y, n=None, incx=1, incy=1):
    x, y = q(x), q(y)
    if n is None:
        n = len(x) // incx
    f = lib().oq_dot_condition
    f.restype = ctypes.c_double
    return f(c_i64(n), P(x), c_i64(incx), P(y), c_i64(incy))


def ulp_err(got, R, r):
    got, R, r = q(got), q(R), q(r)
    out = np.zeros(len(got), dtype=np.float64)
    lib().oq_ulp_err(c_i64(len(got)), P(got), P(R), P(r), P(out))
    return out


def bound_violations(got, ref, absum, kfac):
    got, ref, absum = q(got), q(ref), q(absum)
    return int(lib().oq_count_bound_violations(c_i64(len(got)), P(got), P(ref), P(absum),
                                               ctypes.c_double(kfac)))
