"""quadblas_qdot_dev_noalloc, the qdot entry point for callers that cannot
allocate device memory (their memory belongs to their own allocator or a
fixed plan, or they run latency-sensitive loops that cannot call into the
CUDA allocator).  Its scratch is a static array inside the library, shared
by all calls and left holding the last call's contents.

Checked through the C ABI against quadblas_qdot_dev on two calls in a row,
with the tolerance of the other qdot tests: bit-identical results (both are
the correctly rounded exact sum).  The first call is large (it uses every
block's partial); the second is small, so stale partials left by the first
call would show if they were read.  A second test runs two dots of
condition 1e40 back to back — sums the wide accumulator cannot round alone,
so each arms the exact (Kulisch) pass whose digits live in the static array
— and then a well-conditioned dot: digits left by one exact pass must not
leak into the next, and a certified call must not read a stale exact-pass
flag.  This file is collected last so that a run stopping at the first
failure has already run every other test; it also passes on its own in a
fresh process.
"""
import ctypes

import numpy as np
import pytest

from conftest import to_dev, to_host
from qblas_gb300 import gen as G
from qblas_gb300 import quad as Q

pytestmark = pytest.mark.gpu


def _dot(fn, torch, n, dx, dy, incx=1, incy=1):
    out = torch.zeros((1, 2), dtype=torch.int64, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = fn(n, ctypes.c_void_p(dx.data_ptr()), incx, ctypes.c_void_p(dy.data_ptr()), incy,
            ctypes.c_void_p(out.data_ptr()), stream)
    assert rc == 0, rc
    torch.cuda.synchronize()
    return to_host(out)


def test_noalloc_qdot_matches_qdot_dev_twice(qlib, O, torch_cuda):
    torch = torch_cuda
    rng = G.rng_for(4242)
    cases = [((1 << 22) + 5, 1, 1), (1000, 3, 2)]
    for n, incx, incy in cases:
        x, y = G.cancelling_dot(rng, n * max(incx, incy))
        x, y = x[: n * incx], y[: n * incy]
        dx, dy = to_dev(torch, x), to_dev(torch, y)
        ref = _dot(qlib.quadblas_qdot_dev, torch, n, dx, dy, incx, incy)
        got = _dot(qlib.quadblas_qdot_dev_noalloc, torch, n, dx, dy, incx, incy)
        assert Q.same_bits(got, ref).all(), (n, got, ref)
        R, _, _ = O.exact_dot(x, y, n, incx, incy)
        assert Q.same_bits(got, R).all()


def test_noalloc_exact_pass_twice_then_certified(qlib, O, torch_cuda):
    torch = torch_cuda
    rng = G.rng_for(4343)
    cases = [O.gendot(8192, 1e40, 11), O.gendot(8192, 1e40, 12), G.cancelling_dot(rng, 100003)]
    for i, (x, y) in enumerate(cases):
        n = len(x)
        dx, dy = to_dev(torch, x), to_dev(torch, y)
        got = _dot(qlib.quadblas_qdot_dev_noalloc, torch, n, dx, dy)
        ref = _dot(qlib.quadblas_qdot_dev, torch, n, dx, dy)
        R, _, _ = O.exact_dot(x, y)
        assert Q.same_bits(got, ref).all(), (i, got, ref)
        assert Q.same_bits(got, R).all(), (i, got, R)
    # the two ill-conditioned sums differ, so a stale result would show
    assert not Q.same_bits(O.exact_dot(*cases[0])[0], O.exact_dot(*cases[1])[0]).all()


def test_noalloc_rejects_bad_arguments(qlib, torch_cuda):
    torch = torch_cuda
    d = torch.zeros((4, 2), dtype=torch.int64, device="cuda")
    p = ctypes.c_void_p(d.data_ptr())
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert qlib.quadblas_qdot_dev_noalloc(-1, p, 1, p, 1, p, s) == 1
    assert qlib.quadblas_qdot_dev_noalloc(4, p, 0, p, 1, p, s) == 1
    mis = ctypes.c_void_p(d.data_ptr() + 8)
    assert qlib.quadblas_qdot_dev_noalloc(2, mis, 1, p, 1, p, s) == 6
    # n = 0 is the empty sum, +0
    out = torch.ones((1, 2), dtype=torch.int64, device="cuda")
    assert qlib.quadblas_qdot_dev_noalloc(0, p, 1, p, 1, ctypes.c_void_p(out.data_ptr()), s) == 0
    torch.cuda.synchronize()
    assert Q.same_bits(to_host(out), np.zeros((1, 2), np.uint64)).all()
