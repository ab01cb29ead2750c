"""Seeded synthetic binary128 inputs for each benchmark workload.

All generators return ``(n, 2)`` uint64 binary128 arrays (see ``quad.py``)
and are fully determined by the numpy ``Generator`` they are given.

Workloads (sizes and value distributions):
  * full-mantissa uniform   : a binary64 drawn uniform in [-1, 1) widened to
    binary128, with the 60 significand bits below the binary64 precision
    filled randomly (a random low-order tail below 2^-53 relative), so every
    value has a full 113-bit significand.  Used for the 512^3 soft-float
    qgemm and the batched workload.
  * wide-exponent           : +-u * 2^e, u uniform in [1, 2) with all 112
    fraction bits random, e a uniform integer in [emin, emax] (qdot n=2^26
    and qgemv 8192^2 use [-60, 60]).
  * cancelling dot pairs    : wide-exponent vectors in which half of the
    terms come in pairs whose products cancel to within 2^-80 relative.
  * spread uniform          : u * 2^e with u uniform in [-1, 1) at full
    113-bit significand and e a uniform integer in [emin, emax] (the 4096^3
    Ozaki qgemm uses [-20, 20]).
"""
from __future__ import annotations

import numpy as np

from .quad import BIAS, U64, empty, from_double

_M48 = U64((1 << 48) - 1)
_M60 = U64((1 << 60) - 1)


def rng_for(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def _rand_u64(rng: np.random.Generator, n: int) -> np.ndarray:
    return rng.integers(0, np.iinfo(np.uint64).max, size=n, dtype=np.uint64, endpoint=True)


def uniform_full(rng: np.random.Generator, n: int) -> np.ndarray:
    """Binary64 uniform in [-1, 1) plus a random 60-bit tail below 2^-53."""
    d = rng.uniform(-1.0, 1.0, size=int(n))
    q = from_double(d)
    nz = d != 0
    q[:, 0] = np.where(nz, q[:, 0] | (_rand_u64(rng, d.size) & _M60), q[:, 0])
    return q


def wide_exponent(rng: np.random.Generator, n: int, emin: int = -60, emax: int = 60) -> np.ndarray:
    """+-u * 2^e, u in [1, 2) with 112 random fraction bits, e uniform in [emin, emax]."""
    n = int(n)
    q = empty(n)
    sign = rng.integers(0, 2, size=n, dtype=np.uint64)
    e = rng.integers(emin, emax, size=n, endpoint=True).astype(np.int64)
    bexp = (e + BIAS).astype(np.uint64)
    q[:, 1] = (sign << U64(63)) | (bexp << U64(48)) | (_rand_u64(rng, n) & _M48)
    q[:, 0] = _rand_u64(rng, n)
    return q


def cancelling_dot(rng: np.random.Generator, n: int, emin: int = -60, emax: int = 60):
    """x, y for a dot product in which half of the terms form n/4 pairs whose
    products cancel to within 2^-80 relative (x_b = -x_a perturbed in its
    low 32 significand bits, y_b = y_a), like 1e20 + 1 - 1e20 at scale."""
    x = wide_exponent(rng, n, emin, emax)
    y = wide_exponent(rng, n, emin, emax)
    npairs = n // 4
    if npairs:
        idx = rng.permutation(n)[: 2 * npairs].reshape(npairs, 2)
        a, b = idx[:, 0], idx[:, 1]
        x[b, 1] = x[a, 1] ^ U64(1 << 63)
        x[b, 0] = (x[a, 0] & ~U64(0xFFFFFFFF)) | (_rand_u64(rng, npairs) & U64(0xFFFFFFFF))
        y[b] = y[a]
    return x, y


def spread_uniform(rng: np.random.Generator, n: int, emin: int = -20, emax: int = 20) -> np.ndarray:
    """u * 2^e with u uniform in [-1, 1) (full 113-bit significand) and e
    uniform in [emin, emax]."""
    q = uniform_full(rng, n)
    e = rng.integers(emin, emax, size=int(n), endpoint=True).astype(np.int64)
    bexp = ((q[:, 1] >> U64(48)) & U64(0x7FFF)).astype(np.int64)
    nz = bexp != 0
    nb = np.where(nz, bexp + e, 0).astype(np.uint64)
    q[:, 1] = (q[:, 1] & ~U64(0x7FFF << 48)) | (nb << U64(48))
    return q


def log_uniform_int(rng: np.random.Generator, lo: int, hi: int, n: int) -> np.ndarray:
    """Integers log-uniform in [lo, hi]."""
    v = np.exp(rng.uniform(np.log(lo), np.log(hi + 1), size=int(n)))
    return np.clip(np.floor(v).astype(np.int64), lo, hi)


def uniform_full_device(torch, n: int, seed: int, chunk: int = 1 << 26):
    """uniform_full() generated on the GPU with torch (for multi-GB inputs):
    a binary64 uniform in [-1, 1) widened to binary128 plus a random 60-bit
    tail below 2^-53 relative.  Returns an int64 tensor of shape (n, 2)
    (low word, high word) on the current CUDA device."""
    dev = torch.device("cuda")
    out = torch.empty((int(n), 2), dtype=torch.int64, device=dev)
    g = torch.Generator(device=dev)
    g.manual_seed(int(seed))
    m52 = (1 << 52) - 1
    for s in range(0, int(n), chunk):
        e = min(int(n), s + chunk)
        d = torch.rand(e - s, dtype=torch.float64, device=dev, generator=g) * 2.0 - 1.0
        bits = d.view(torch.int64)
        sign = (bits >> 63) & 1
        ex = (bits >> 52) & 0x7FF
        frac = bits & m52
        hi = (sign << 63) | ((ex - 1023 + 16383) << 48) | (frac >> 4)
        tail = torch.randint(0, 1 << 60, (e - s,), dtype=torch.int64, device=dev, generator=g)
        lo = ((frac & 0xF) << 60) | tail
        zero = d == 0
        out[s:e, 0] = torch.where(zero, torch.zeros_like(lo), lo)
        out[s:e, 1] = torch.where(zero, sign << 63, hi)
    return out


def config4_shapes(rng: np.random.Generator, count: int = 10000):
    """Shapes of the batched workload: `count` qgemm problems with m, n, k
    log-uniform in [8, 256], `count` qgemv problems with m, n log-uniform in
    [16, 2048] and `count` qdot problems with n log-uniform in [64, 65536].
    Returns (gemm (count, 3) [m, n, k], gemv (count, 2) [m, n], dot (count,))."""
    gm = log_uniform_int(rng, 8, 256, 3 * count).reshape(3, count).T.copy()
    gv = log_uniform_int(rng, 16, 2048, 2 * count).reshape(2, count).T.copy()
    dn = log_uniform_int(rng, 64, 65536, count)
    return gm, gv, dn


def config4_batch(torch, seed: int):
    """The batched workload on the current CUDA device: config4_shapes(seed)
    with full-mantissa uniform values, row-major 'N', alpha = 1, beta = 0.
    Returns (problems, inputs, outputs, layout): `problems` a PROBLEM_DTYPE
    array for quadblas_batch_plan; A and B of every problem in the device
    tensor `inputs`, C in `outputs` (both (count, 2) int64, uniform_full
    values); layout[i] = (op, m, n, k, offset of A, of B, of C, length of C)
    in elements."""
    from .api import PROBLEM_DTYPE
    from .quad import scalar
    gm, gv, dn = config4_shapes(rng_for(seed))
    lay = []
    oi = oo = 0
    for m, n, k in gm:
        lay.append((0, int(m), int(n), int(k), oi, oi + m * k, oo, int(m * n)))
        oi += m * k + k * n
        oo += m * n
    for m, n in gv:
        lay.append((1, int(m), int(n), 0, oi, oi + m * n, oo, int(m)))
        oi += m * n + n
        oo += m
    for n in dn:
        lay.append((2, 0, int(n), 0, oi, oi + n, oo, 1))
        oi += 2 * n
        oo += 1
    inp = uniform_full_device(torch, int(oi), seed=seed + 1)
    out = uniform_full_device(torch, int(oo), seed=seed + 2)
    bi, bo = inp.data_ptr(), out.data_ptr()
    probs = np.zeros(len(lay), dtype=PROBLEM_DTYPE)
    one, zero = scalar(1.0)[0], scalar(0.0)[0]
    for p, (op, m, n, k, a, b, c, _) in zip(probs, lay):
        p["op"], p["layout"], p["transa"], p["transb"] = op, b"R", b"N", b"N"
        p["m"], p["n"], p["k"] = m, n, k
        p["alpha"], p["beta"] = one, zero
        p["A"], p["B"], p["C"] = bi + 16 * int(a), bi + 16 * int(b), bo + 16 * int(c)
        if op == 0:
            p["lda"], p["ldb"], p["ldc"] = k, n, n
        elif op == 1:
            p["lda"], p["ldb"], p["ldc"] = n, 1, 1
        else:
            p["lda"], p["ldb"], p["ldc"] = 1, 1, 1
    return probs, inp, out, lay
