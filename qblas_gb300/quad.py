"""IEEE binary128 values held as numpy ``uint64`` pairs.

A binary128 array of n elements is an ``(n, 2)`` uint64 array: column 0 is
the low 64 bits of the significand, column 1 holds the sign (bit 63), the
15-bit biased exponent (bits 62..48) and the high 48 significand bits.  This
is the in-memory layout of ``Sleef_quad`` (and of ``__float128`` /
AArch64 ``long double``) on little-endian hosts, so these arrays can be
passed straight to the C ABI (``void *`` of ``Sleef_quad``).
"""
from __future__ import annotations

import numpy as np

U64 = np.uint64
BIAS = 16383
_M52 = U64((1 << 52) - 1)
_M48 = U64((1 << 48) - 1)


def empty(n: int) -> np.ndarray:
    return np.zeros((int(n), 2), dtype=np.uint64)


def as_quad(a) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.uint64)
    if a.ndim != 2 or a.shape[1] != 2:
        raise ValueError("binary128 arrays are (n, 2) uint64")
    return a


def longdouble_is_binary128() -> bool:
    """True where numpy's longdouble is IEEE binary128 (AArch64 Linux), so
    that its arrays hold binary128 values as they are."""
    fi = np.finfo(np.longdouble)
    return np.dtype(np.longdouble).itemsize == 16 and fi.nmant == 112 and fi.maxexp == 16384


def view(a) -> np.ndarray:
    """A zero-copy ``(n, 2)`` uint64 view of a buffer of binary128 values, so
    that outputs written through it land in the caller's memory:

    * ``(n, 2)`` (or ``(..., 2)``) uint64 arrays, as they are;
    * numpy arrays of any 16-byte dtype that holds binary128 values: ``V16``,
      a binary128 quad-precision dtype exposing the buffer protocol, or
      ``longdouble`` where it is binary128 (``longdouble_is_binary128``;
      elsewhere it is the x87 80-bit format, which is refused);
    * any other object exporting a contiguous buffer of 16-byte items.

    Non-contiguous buffers are refused rather than copied."""
    if isinstance(a, np.ndarray):
        if a.dtype == np.uint64 and a.ndim >= 1 and a.shape[-1] == 2:
            if not a.flags.c_contiguous:
                raise ValueError("binary128 arrays must be C-contiguous")
            return a.reshape(-1, 2)
        if a.dtype.itemsize != 16:
            raise ValueError(f"dtype {a.dtype} does not hold binary128 values (16 bytes per element)")
        if a.dtype == np.longdouble and not longdouble_is_binary128():
            raise ValueError("numpy longdouble is not binary128 on this platform")
        if a.dtype.kind in "iufc" and a.dtype != np.longdouble:
            raise ValueError(f"dtype {a.dtype} does not hold binary128 values")
        if not a.flags.c_contiguous:
            raise ValueError("binary128 arrays must be C-contiguous")
        return a.reshape(-1).view(np.uint64).reshape(-1, 2)
    mv = memoryview(a)
    if mv.itemsize != 16 and not (mv.itemsize == 1 and mv.nbytes % 16 == 0 and mv.format in ("B", "b", "c")):
        raise ValueError("buffer items are not 16-byte binary128 values")
    if not mv.c_contiguous:
        raise ValueError("binary128 buffers must be contiguous")
    return np.frombuffer(mv.cast("B"), dtype=np.uint64).reshape(-1, 2)


def from_double(d) -> np.ndarray:
    """Exact binary64 -> binary128 widening (what Sleef_cast_from_doubleq1 does)."""
    d = np.ascontiguousarray(d, dtype=np.float64).ravel()
    out = empty(d.size)
    bits = d.view(np.uint64)
    sign = bits >> U64(63)
    fin = np.isfinite(d) & (d != 0)
    m, e = np.frexp(np.abs(np.where(fin, d, 1.0)))  # |d| = m * 2^e, m in [0.5, 1)
    M = (m * 2.0**53).astype(np.uint64)
    bexp = (e.astype(np.int64) - 1 + BIAS).astype(np.uint64)
    frac = M & _M52
    hi = (sign << U64(63)) | (bexp << U64(48)) | (frac >> U64(4))
    lo = (frac & U64(0xF)) << U64(60)
    hi = np.where(fin, hi, sign << U64(63))
    lo = np.where(fin, lo, U64(0))
    inf = np.isinf(d)
    hi = np.where(inf, (sign << U64(63)) | U64(0x7FFF000000000000), hi)
    nan = np.isnan(d)
    hi = np.where(nan, U64(0x7FFF800000000000), hi)
    out[:, 0] = lo
    out[:, 1] = hi
    return out


def to_double_approx(q) -> np.ndarray:
    """binary128 -> float64 by truncation (for display and coarse checks only)."""
    q = as_quad(q)
    hi = q[:, 1]
    sign = np.where((hi >> U64(63)) != 0, -1.0, 1.0)
    bexp = ((hi >> U64(48)) & U64(0x7FFF)).astype(np.int64)
    frac = (hi & _M48).astype(np.float64) * 2.0**-48 + (q[:, 0] >> U64(11)).astype(np.float64) * 2.0**-101
    normal = bexp != 0
    val = np.where(normal, 1.0 + frac, frac)
    ex = np.where(normal, bexp - BIAS, -16382)
    with np.errstate(over="ignore", under="ignore"):
        out = sign * np.ldexp(val, np.clip(ex, -2000, 2000).astype(np.int64))
    special = bexp == 0x7FFF
    isnan = special & (((hi & _M48) | q[:, 0]) != 0)
    out = np.where(special, sign * np.inf, out)
    out = np.where(isnan, np.nan, out)
    return out


def is_nan(q) -> np.ndarray:
    q = as_quad(q)
    hi = q[:, 1]
    return (((hi >> U64(48)) & U64(0x7FFF)) == U64(0x7FFF)) & (((hi & _M48) | q[:, 0]) != 0)


def same_bits(a, b) -> np.ndarray:
    """Elementwise bit equality, treating any two NaNs as equal."""
    a, b = as_quad(a), as_quad(b)
    eq = (a[:, 0] == b[:, 0]) & (a[:, 1] == b[:, 1])
    return eq | (is_nan(a) & is_nan(b))


def scalar(x: float) -> np.ndarray:
    return from_double(np.array([x]))
