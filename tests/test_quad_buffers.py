"""The binding's binary128 buffer adapter (quad.view): the Python/numpy
integration that include/quadblas/interface/c_interface.hpp:13 anticipates.
Every accepted buffer is viewed in place (outputs land in the caller's
memory); buffers that do not hold binary128 values, and non-contiguous ones,
are refused instead of being converted or copied."""
import numpy as np
import pytest

from qblas_gb300 import api
from qblas_gb300 import quad as Q
from qblas_gb300._lib import QblasError


def test_uint64_pairs_are_used_in_place():
    a = Q.from_double([1.0, -2.5, 3.25])
    v = Q.view(a)
    assert v.shape == (3, 2) and np.shares_memory(v, a)
    assert Q.view(a.reshape(1, 3, 2)).shape == (3, 2)


def test_v16_and_raw_buffers():
    ref = Q.from_double([0.5, -7.0, 1e300, -0.0])
    v16 = ref.copy().view(np.dtype("V16")).reshape(-1)
    assert v16.dtype.itemsize == 16 and v16.shape == (4,)
    w = Q.view(v16)
    assert np.shares_memory(w, v16) and Q.same_bits(w, ref).all()
    raw = bytearray(ref.tobytes())
    w2 = Q.view(raw)
    assert Q.same_bits(w2, ref).all()
    w2[1] = Q.from_double([42.0])[0]  # writes reach the caller's buffer
    assert Q.same_bits(np.frombuffer(bytes(raw), dtype=np.uint64).reshape(-1, 2)[1:2], Q.from_double([42.0])).all()


def test_longdouble_only_where_it_is_binary128():
    ld = np.array([1.5, -2.25, 3.0], dtype=np.longdouble)
    if Q.longdouble_is_binary128():
        assert Q.same_bits(Q.view(ld), Q.from_double([1.5, -2.25, 3.0])).all()
    else:
        with pytest.raises(ValueError):
            Q.view(ld)


def test_refused_buffers():
    with pytest.raises(ValueError):
        Q.view(np.zeros(4, dtype=np.float64))
    with pytest.raises(ValueError):
        Q.view(np.zeros((8, 2), dtype=np.uint64)[::2])
    with pytest.raises(ValueError):
        Q.view(np.zeros(3, dtype=np.complex128))
    with pytest.raises(ValueError):
        Q.view(bytearray(24))


def test_entry_points_take_the_buffers(qlib):
    """A V16 array reaches the library (which, without a GPU, then reports
    that there is none) rather than being refused or converted by the
    binding."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present: test_buffers_on_the_gpu_path covers the calls")
    except ImportError:
        pass
    x = Q.from_double(np.arange(1.0, 5.0)).view(np.dtype("V16")).reshape(-1)
    with pytest.raises(QblasError):
        api.dot(x, x)
    with pytest.raises(QblasError):
        api.gemv("R", "N", 2, 2, 1.0, x, 2, x[:2], 1, 0.0, x[2:], 1)


@pytest.mark.gpu
def test_buffers_on_the_gpu_path(qlib, O, torch_cuda):
    """qdot, qgemv and qgemm on V16 arrays (and on numpy longdouble arrays
    where longdouble is binary128, as on AArch64 hosts) give the same bits
    as on (n, 2) uint64 arrays, with the outputs written in place."""
    from qblas_gb300 import gen as G
    rng = G.rng_for(91)
    m, n, k = 33, 20, 47
    A, B, C = G.uniform_full(rng, m * k), G.uniform_full(rng, k * n), G.uniform_full(rng, m * n)
    x, y = G.uniform_full(rng, k), G.uniform_full(rng, m)
    ref_d = api.dot(A[:k], x)
    yr, Cr = y.copy(), C.copy()
    api.gemv("R", "N", m, k, 1.5, A, k, x, 1, 0.5, yr, 1)
    api.gemm("R", "N", "N", m, n, k, 2.0, A, k, B, n, -1.0, Cr, n)
    kinds = [lambda a: a.copy().view(np.dtype("V16")).reshape(-1)]
    if Q.longdouble_is_binary128():
        kinds.append(lambda a: a.copy().view(np.longdouble).reshape(-1))
    for mk in kinds:
        A2, B2, x2, y2, C2 = mk(A), mk(B), mk(x), mk(y), mk(C)
        assert Q.same_bits(api.dot(A2[:k], x2), ref_d).all()
        api.gemv("R", "N", m, k, 1.5, A2, k, x2, 1, 0.5, y2, 1)
        assert Q.same_bits(Q.view(y2), yr).all()
        api.gemm("R", "N", "N", m, n, k, 2.0, A2, k, B2, n, -1.0, C2, n)
        assert Q.same_bits(Q.view(C2), Cr).all()
