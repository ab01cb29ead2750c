"""Device-side bounded waits that run out, made on purpose without stalling
the GPU (quadblas_debug_stall_next_call): the next Ozaki kernel withholds one
accumulator-full commit (an arrive; no copy is withheld) and shortens its
pipeline waits to 1 ms.  Its epilogue's wait then runs out, the other roles
run out after it, every copy and tensor-core operation in flight is waited
for with the standard 1 s limit, and the kernel frees its tensor memory and
returns.  The reference has no equivalent: its CPU calls cannot time out.

* qgemm (one 128 x 256 tile, one k block): the host-pointer call returns
  QBLAS_ERR_TIMEOUT with NaN in C; the device-pointer call returns after
  enqueueing and the device flag (quadblas_device_status) reports the
  timeout; the next calls are bit-identical to the same call made before.
* qgemv: the row finish sends every row to the exact pass (the exact-row
  counter shows all of them), so the results stay correctly rounded.
"""
import ctypes

import numpy as np
import pytest

from conftest import to_dev, to_host
from gpu_helpers import epilogue
from qblas_gb300 import api
from qblas_gb300 import gen as G
from qblas_gb300 import quad as Q

pytestmark = pytest.mark.gpu
TIMEOUT = 7


def P(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def is_nan(q):
    q = Q.as_quad(q)
    return (((q[:, 1] >> np.uint64(48)) & np.uint64(0x7FFF)) == 0x7FFF) & \
        (((q[:, 1] & np.uint64((1 << 48) - 1)) | q[:, 0]) != 0)


@pytest.fixture
def ozaki(qlib):
    api.set_method(2)
    yield qlib
    api.set_method(0)
    qlib.quadblas_device_status(1)


def test_qgemm_timeout_reported_then_recovered(ozaki, O, torch_cuda):
    qlib, torch = ozaki, torch_cuda
    m, n, k = 128, 256, 64
    rng = G.rng_for(808)
    A, B = G.spread_uniform(rng, m * k), G.spread_uniform(rng, k * n)
    one, zero = Q.scalar(1.0), Q.scalar(0.0)

    def host_call():
        C = Q.from_double(np.zeros(m * n))
        rc = qlib.quadblas_qgemm_q(b"R", b"N", b"N", m, n, k, P(one), P(A), k, P(B), n, P(zero), P(C), n)
        return rc, C

    rc, ref = host_call()
    assert rc == 0 and not is_nan(ref).any()
    assert qlib.quadblas_debug_stall_next_call(1) == 0
    rc, got = host_call()
    assert rc == TIMEOUT
    assert is_nan(got).all()
    rc, again = host_call()
    assert rc == 0 and Q.same_bits(again, ref).all()

    # device pointers: the call returns after enqueueing; the flag tells
    dA, dB = to_dev(torch, A), to_dev(torch, B)
    dC = torch.zeros((m * n, 2), dtype=torch.int64, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def dev_call():
        dC.zero_()
        rc = qlib.quadblas_qgemm_dev(b"R", b"N", b"N", m, n, k, P(one), ctypes.c_void_p(dA.data_ptr()), k,
                                     ctypes.c_void_p(dB.data_ptr()), n, P(zero), ctypes.c_void_p(dC.data_ptr()), n,
                                     stream)
        torch.cuda.synchronize()
        return rc, to_host(dC)

    assert qlib.quadblas_device_status(1) == 0
    assert qlib.quadblas_debug_stall_next_call(1) == 0
    rc, got = dev_call()
    assert rc == 0
    assert is_nan(got).all()
    assert qlib.quadblas_device_status(1) == TIMEOUT
    assert qlib.quadblas_device_status(0) == 0  # cleared by the read above
    rc, again = dev_call()
    assert rc == 0 and Q.same_bits(again, ref).all()
    assert qlib.quadblas_device_status(1) == 0


def test_qgemv_timeout_recomputes_every_row(ozaki, O, torch_cuda):
    qlib, torch = ozaki, torch_cuda
    m, n = 300, 512
    rng = G.rng_for(809)
    A, x = G.wide_exponent(rng, m * n), G.wide_exponent(rng, n)
    y0 = G.wide_exponent(rng, m)
    al, be = Q.scalar(1.5), Q.scalar(0.5)
    R, _, _ = O.exact_gemv(m, n, A, n, 1, x, 1)
    want = epilogue(O, al, R, be, y0)
    api.debug_count_exact_rows(True)
    try:
        assert qlib.quadblas_debug_stall_next_call(2) == 0
        y = y0.copy()
        api.gemv("R", "N", m, n, al, A, n, x, 1, be, y, 1)
        assert Q.same_bits(y, want).all()
        assert api.debug_exact_rows() == m  # every row went through the exact pass
        y = y0.copy()
        api.gemv("R", "N", m, n, al, A, n, x, 1, be, y, 1)
        assert Q.same_bits(y, want).all()
        assert api.debug_exact_rows() < m  # a normal call certifies most rows
    finally:
        api.debug_count_exact_rows(False)
