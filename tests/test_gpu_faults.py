"""Failure handling under injected allocation failures (host-side fault
injection: quadblas_debug_fail_allocations makes the library's next device
allocations fail as if the device were out of memory; no GPU fault is
involved).  Every entry point that needs device memory must return
QBLAS_ERR_NO_MEMORY, leave its outputs untouched, record the status for
quadblas_last_error, and work normally on the next call."""
import ctypes

import numpy as np
import pytest

from conftest import to_dev, to_host
from qblas_gb300 import api
from qblas_gb300 import gen as G
from qblas_gb300 import quad as Q

pytestmark = pytest.mark.gpu
NO_MEMORY = 3


def P(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def dptr(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.fixture
def faults(qlib):
    yield qlib
    qlib.quadblas_debug_fail_allocations(0)
    api.set_method(0)


def test_device_pointer_paths(faults, O, torch_cuda):
    qlib, torch = faults, torch_cuda
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = G.rng_for(61)
    n = 5000
    x, y = G.uniform_full(rng, n), G.uniform_full(rng, n)
    dx, dy = to_dev(torch, x), to_dev(torch, y)
    sentinel = Q.scalar(7.0)
    dres = to_dev(torch, sentinel)
    qlib.quadblas_debug_fail_allocations(1)
    assert qlib.quadblas_qdot_dev(n, dptr(dx), 1, dptr(dy), 1, dptr(dres), s) == NO_MEMORY
    assert qlib.quadblas_last_error() == NO_MEMORY
    torch.cuda.synchronize()
    assert Q.same_bits(to_host(dres), sentinel).all()
    assert qlib.quadblas_qdot_dev(n, dptr(dx), 1, dptr(dy), 1, dptr(dres), s) == 0
    torch.cuda.synchronize()
    R, _, _ = O.exact_dot(x, y)
    assert Q.same_bits(to_host(dres), R).all()

    m, k = 40, 300
    A = G.uniform_full(rng, m * k)
    dA, dv = to_dev(torch, A), to_dev(torch, x[:k])
    yold = G.uniform_full(rng, m)
    dy2 = to_dev(torch, yold)
    one, zero = Q.scalar(1.0), Q.scalar(0.0)
    qlib.quadblas_debug_fail_allocations(1)
    assert qlib.quadblas_qgemv_dev(b"R", b"N", m, k, P(one), dptr(dA), k, dptr(dv), 1, P(zero), dptr(dy2), 1,
                                   s) == NO_MEMORY
    torch.cuda.synchronize()
    assert Q.same_bits(to_host(dy2), yold).all()
    assert qlib.quadblas_qgemv_dev(b"R", b"N", m, k, P(one), dptr(dA), k, dptr(dv), 1, P(zero), dptr(dy2), 1,
                                   s) == 0

    # Ozaki qgemm takes its digit planes from the pool; soft-float qgemm needs no scratch
    B = G.uniform_full(rng, k * m)
    C0 = G.uniform_full(rng, m * m)
    dB, dC = to_dev(torch, B), to_dev(torch, C0)
    api.set_method(2)
    qlib.quadblas_debug_fail_allocations(1)
    assert qlib.quadblas_qgemm_dev(b"R", b"N", b"N", m, m, k, P(one), dptr(dA), k, dptr(dB), m, P(zero),
                                   dptr(dC), m, s) == NO_MEMORY
    torch.cuda.synchronize()
    assert Q.same_bits(to_host(dC), C0).all()
    assert qlib.quadblas_qgemm_dev(b"R", b"N", b"N", m, m, k, P(one), dptr(dA), k, dptr(dB), m, P(zero),
                                   dptr(dC), m, s) == 0


def test_host_pointer_paths(faults, O):
    qlib = faults
    rng = G.rng_for(62)
    n = 3000
    x, y = G.uniform_full(rng, n), G.uniform_full(rng, n)
    res = Q.scalar(7.0).copy()
    api.release_buffers()  # the next host-pointer call has to allocate its staging buffers
    qlib.quadblas_debug_fail_allocations(1)
    assert qlib.quadblas_qdot_q(n, P(x), 1, P(y), 1, P(res)) == NO_MEMORY
    assert Q.same_bits(res, Q.scalar(7.0)).all()
    assert qlib.quadblas_qdot_q(n, P(x), 1, P(y), 1, P(res)) == 0
    R, _, _ = O.exact_dot(x, y)
    assert Q.same_bits(res, R).all()

    # the reference's void qgemm reports through quadblas_last_error
    m, k = 30, 50
    A, B = G.uniform_full(rng, m * k), G.uniform_full(rng, k * m)
    C0 = G.uniform_full(rng, m * m)
    C = C0.copy()
    api.release_buffers()
    qlib.quadblas_debug_fail_allocations(1)
    qlib.quadblas_qgemm(b"R", b"N", b"N", m, m, k, ctypes.c_double(1.0), P(A), k, P(B), m, ctypes.c_double(0.0),
                        P(C), m)
    assert qlib.quadblas_last_error() == NO_MEMORY
    assert Q.same_bits(C, C0).all()
    qlib.quadblas_qgemm(b"R", b"N", b"N", m, m, k, ctypes.c_double(1.0), P(A), k, P(B), m, ctypes.c_double(0.0),
                        P(C), m)
    assert qlib.quadblas_last_error() == 0
    rows, cols = np.meshgrid(np.arange(m), np.arange(m), indexing="ij")
    R, _, _ = O.exact_gemm(k, A, k, 1, B, m, 1, rows.ravel(), cols.ravel())
    assert Q.same_bits(C, R).all()


def test_batch_plan(faults, torch_cuda):
    qlib, torch = faults, torch_cuda
    rng = G.rng_for(63)
    x, y = G.uniform_full(rng, 100), G.uniform_full(rng, 100)
    buf = to_dev(torch, np.concatenate([x, y, Q.scalar(0.0)]))
    base = buf.data_ptr()
    probs = np.zeros(1, dtype=api.PROBLEM_DTYPE)
    p = probs[0]
    p["op"], p["layout"], p["transa"], p["transb"] = 2, b"R", b"N", b"N"
    p["n"], p["lda"], p["ldb"], p["ldc"] = 100, 1, 1, 1
    p["A"], p["B"], p["C"] = base, base + 16 * 100, base + 16 * 200
    p["alpha"], p["beta"] = Q.scalar(1.0)[0], Q.scalar(0.0)[0]
    h = ctypes.c_void_p()
    qlib.quadblas_debug_fail_allocations(1)
    assert qlib.quadblas_batch_plan(P(probs), 1, ctypes.byref(h)) == NO_MEMORY
    assert not h.value
    plan = api.BatchPlan(probs)  # allocation works again
    plan.execute()
    torch.cuda.synchronize()
    plan.close()
