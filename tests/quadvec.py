"""Binary128 test-vector generators for the elementwise soft-float checks:
random bit patterns, narrow-exponent values (cancellation), sparse
significands (rounding ties), subnormals, overflow/underflow edges and the
special values."""
from __future__ import annotations

import numpy as np

U64 = np.uint64
M48 = U64((1 << 48) - 1)


def _u64(rng, n):
    return rng.integers(0, np.iinfo(np.uint64).max, size=n, dtype=np.uint64, endpoint=True)


def specials() -> np.ndarray:
    v = [
        (0, 0), (0, 1 << 63),                                  # +0, -0
        (0, 0x7FFF << 48), (0, (0x7FFF << 48) | (1 << 63)),     # +inf, -inf
        (0, 0x7FFF8 << 44),                                    # qNaN
        (1, 0), (1, 1 << 63),                                  # smallest subnormals
        ((1 << 64) - 1, (1 << 48) - 1),                        # largest subnormal
        (0, 1 << 48),                                          # smallest normal
        ((1 << 64) - 1, (0x7FFE << 48) | ((1 << 48) - 1)),     # largest finite
        (0, 0x3FFF << 48), (0, (0x3FFF << 48) | (1 << 63)),    # +1, -1
        (0, 0x4000 << 48), (0, 0x3FFE << 48),                  # 2, 0.5
        (1, 0x3FFF << 48),                                     # 1 + 2^-112
        ((1 << 64) - 1, (0x3FFE << 48) | ((1 << 48) - 1)),     # 1 - 2^-113
    ]
    return np.array(v, dtype=np.uint64)


def random_bits(rng, n) -> np.ndarray:
    return np.stack([_u64(rng, n), _u64(rng, n)], axis=1)


def finite(rng, n, emin=-16382, emax=16383, sparse=False) -> np.ndarray:
    """Finite normal values with biased exponent drawn from [emin, emax] + bias."""
    q = np.zeros((n, 2), dtype=np.uint64)
    sign = rng.integers(0, 2, size=n, dtype=np.uint64)
    e = rng.integers(emin, emax, size=n, endpoint=True) + 16383
    e = np.clip(e, 1, 0x7FFE).astype(np.uint64)
    if sparse:
        # few set bits: top 6 and bottom 6 bits of the fraction
        hi_f = (rng.integers(0, 64, size=n, dtype=np.uint64) << U64(42))
        lo_f = rng.integers(0, 64, size=n, dtype=np.uint64)
        q[:, 1] = (sign << U64(63)) | (e << U64(48)) | hi_f
        q[:, 0] = lo_f
    else:
        q[:, 1] = (sign << U64(63)) | (e << U64(48)) | (_u64(rng, n) & M48)
        q[:, 0] = _u64(rng, n)
    return q


def subnormal(rng, n) -> np.ndarray:
    q = np.zeros((n, 2), dtype=np.uint64)
    sign = rng.integers(0, 2, size=n, dtype=np.uint64)
    shift = rng.integers(0, 112, size=n)
    hi = _u64(rng, n) & M48
    lo = _u64(rng, n)
    # thin out leading bits so that all subnormal magnitudes appear
    mh = np.where(shift >= 48, U64(0), hi >> np.minimum(shift, 47).astype(np.uint64))
    ml = np.where(shift >= 48, lo >> np.minimum(shift - 48, 63).clip(0).astype(np.uint64), lo)
    q[:, 1] = (sign << U64(63)) | mh
    q[:, 0] = ml
    return q


def mixed(rng, n) -> np.ndarray:
    """A mixture of all of the above, shuffled."""
    parts = [
        random_bits(rng, n // 8),
        finite(rng, n // 4, -40, 40),
        finite(rng, n // 8, -40, 40, sparse=True),
        finite(rng, n // 8),
        finite(rng, n // 16, -16382, -16200),
        finite(rng, n // 16, 16200, 16383),
        subnormal(rng, n // 8),
    ]
    got = sum(len(p) for p in parts)
    sp = specials()
    reps = np.resize(sp, (max(n - got, 0), 2))
    allv = np.concatenate(parts + [reps])[:n]
    return allv[rng.permutation(len(allv))]
