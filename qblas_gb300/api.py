"""Python front end of the C ABI, mirroring the reference's C interface
(include/quadblas/interface/c_interface.hpp) argument for argument.

Host functions take binary128 buffers — numpy ``(n, 2)`` uint64 arrays (see
``quad.py``), arrays of a 16-byte binary128 dtype (numpy's longdouble where
it is binary128, a quad-precision dtype exposing the buffer protocol,
``V16``), or any contiguous buffer of 16-byte items — viewed without a copy
(``quad.view``), and update outputs in place, like the C calls.  Device
functions take CUDA tensors whose storage holds binary128 values (any
dtype; 16 bytes per element, e.g. int64 of shape (n, 2)) and an optional
CUDA stream (defaults to torch's current stream)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import quad
from ._lib import check, load


def _p(a):
    """Address of a binary128 buffer (viewed in place, never copied)."""
    return quad.view(a).ctypes.data_as(ctypes.c_void_p)


def _q1(v) -> np.ndarray:
    """A binary128 scalar: a Python number (widened exactly from binary64), a
    (1, 2) uint64 array, or a 16-byte binary128 value (e.g. numpy longdouble
    where it is binary128)."""
    if isinstance(v, (float, int)):
        return quad.scalar(float(v))
    if isinstance(v, np.ndarray) and v.dtype == np.uint64:
        return quad.as_quad(v)
    if isinstance(v, np.generic):
        v = np.asarray(v).reshape(1)
    return np.ascontiguousarray(quad.view(v))


def _c(ch: str) -> bytes:
    return ch.encode()[:1]


# ---- reference-compatible (double scalars, host pointers) ---------------
def qdot(n, x, incx, y, incy) -> float:
    return load().quadblas_qdot(n, _p(x), incx, _p(y), incy)


def qnrm2(n, x, incx) -> float:
    return load().quadblas_qnrm2(n, _p(x), incx)


def qaxpy(n, alpha: float, x, incx, y, incy) -> None:
    load().quadblas_qaxpy(n, alpha, _p(x), incx, _p(y), incy)


def qgemv(layout, trans, m, n, alpha: float, A, lda, x, incx, beta: float, y, incy) -> None:
    load().quadblas_qgemv(_c(layout), _c(trans), m, n, alpha, _p(A), lda, _p(x), incx, beta, _p(y), incy)


def qgemm(layout, transa, transb, m, n, k, alpha: float, A, lda, B, ldb, beta: float, C, ldc) -> None:
    load().quadblas_qgemm(_c(layout), _c(transa), _c(transb), m, n, k, alpha, _p(A), lda, _p(B), ldb,
                          beta, _p(C), ldc)


# ---- binary128 results and scalars (host pointers) ----------------------
def dot(x, y, n=None, incx=1, incy=1) -> np.ndarray:
    x, y = quad.view(x), quad.view(y)
    if n is None:
        n = len(x) // incx
    out = quad.empty(1)
    check(load().quadblas_qdot_q(n, _p(x), incx, _p(y), incy, _p(out)))
    return out


def nrm2(x, n=None, incx=1) -> np.ndarray:
    x = quad.view(x)
    if n is None:
        n = len(x) // incx
    out = quad.empty(1)
    check(load().quadblas_qnrm2_q(n, _p(x), incx, _p(out)))
    return out


def axpy(alpha, x, y, n=None, incx=1, incy=1) -> None:
    x, y, a = quad.view(x), quad.view(y), _q1(alpha)
    if n is None:
        n = len(x) // incx
    check(load().quadblas_qaxpy_q(n, _p(a), _p(x), incx, _p(y), incy))


def gemv(layout, trans, m, n, alpha, A, lda, x, incx, beta, y, incy) -> None:
    a, b = _q1(alpha), _q1(beta)
    check(load().quadblas_qgemv_q(_c(layout), _c(trans), m, n, _p(a), _p(A), lda, _p(x), incx, _p(b),
                                  _p(y), incy))


def gemm(layout, transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc) -> None:
    a, b = _q1(alpha), _q1(beta)
    check(load().quadblas_qgemm_q(_c(layout), _c(transa), _c(transb), m, n, k, _p(a), _p(A), lda, _p(B),
                                  ldb, _p(b), _p(C), ldc))


# ---- device pointers ------------------------------------------------------
def _stream(stream):
    if stream is None:
        import torch
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    if isinstance(stream, int):
        return ctypes.c_void_p(stream)
    return ctypes.c_void_p(stream.cuda_stream)


def _dp(t):
    return ctypes.c_void_p(t.data_ptr())


def dot_dev(n, dx, incx, dy, incy, dres, stream=None) -> None:
    check(load().quadblas_qdot_dev(n, _dp(dx), incx, _dp(dy), incy, _dp(dres), _stream(stream)))


def nrm2_dev(n, dx, incx, dres, stream=None) -> None:
    check(load().quadblas_qnrm2_dev(n, _dp(dx), incx, _dp(dres), _stream(stream)))


def axpy_dev(n, alpha, dx, incx, dy, incy, stream=None) -> None:
    a = _q1(alpha)
    check(load().quadblas_qaxpy_dev(n, _p(a), _dp(dx), incx, _dp(dy), incy, _stream(stream)))


def gemv_dev(layout, trans, m, n, alpha, dA, lda, dx, incx, beta, dy, incy, stream=None) -> None:
    a, b = _q1(alpha), _q1(beta)
    check(load().quadblas_qgemv_dev(_c(layout), _c(trans), m, n, _p(a), _dp(dA), lda, _dp(dx), incx,
                                    _p(b), _dp(dy), incy, _stream(stream)))


def gemm_dev(layout, transa, transb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc, stream=None) -> None:
    a, b = _q1(alpha), _q1(beta)
    check(load().quadblas_qgemm_dev(_c(layout), _c(transa), _c(transb), m, n, k, _p(a), _dp(dA), lda,
                                    _dp(dB), ldb, _p(b), _dp(dC), ldc, _stream(stream)))


def set_method(method: int) -> None:
    check(load().quadblas_set_method(method))


def set_ozaki_slices(s: int) -> None:
    check(load().quadblas_set_ozaki_slices(s))


def set_ozaki_digit_bits(b: int) -> None:
    check(load().quadblas_set_ozaki_digit_bits(b))


def set_ozaki_scheme(scheme: int) -> None:
    """0 automatic (residues when they fit), 1 digit pairs, 2 residues (CRT)."""
    check(load().quadblas_set_ozaki_scheme(scheme))


def get_ozaki_scheme() -> int:
    return load().quadblas_get_ozaki_scheme()


def device_status(clear: bool = True) -> int:
    """QBLAS_ERR_TIMEOUT (7) if a device-pointer Ozaki qgemm on the current
    device timed out since the last clear, else 0 (read after syncing)."""
    return int(load().quadblas_device_status(1 if clear else 0))


def release_buffers() -> None:
    check(load().quadblas_release_buffers())


def debug_fail_allocations(count: int) -> None:
    check(load().quadblas_debug_fail_allocations(count))


def debug_count_exact_rows(on: bool) -> None:
    check(load().quadblas_debug_count_exact_rows(1 if on else 0))


def debug_exact_rows() -> int:
    """Rows the last qgemv recomputed exactly (after its stream completed)."""
    return int(load().quadblas_debug_exact_rows())


# ---- batched problems (one persistent launch) -------------------------------
OP_GEMM, OP_GEMV, OP_DOT = 0, 1, 2

PROBLEM_DTYPE = np.dtype([("op", "<i4"), ("layout", "S1"), ("transa", "S1"), ("transb", "S1"),
                          ("reserved", "S1"), ("m", "<i8"), ("n", "<i8"), ("k", "<i8"),
                          ("alpha", "<u8", (2,)), ("beta", "<u8", (2,)), ("A", "<u8"), ("lda", "<i8"),
                          ("B", "<u8"), ("ldb", "<i8"), ("C", "<u8"), ("ldc", "<i8")], align=True)
assert PROBLEM_DTYPE.itemsize == 112


def batched_dev(problems: np.ndarray, stream=None) -> None:
    """One batch, once (quadblas_qgemm_batched_dev): plan, execute, wait, free."""
    problems = np.ascontiguousarray(problems, dtype=PROBLEM_DTYPE)
    check(load().quadblas_qgemm_batched_dev(problems.ctypes.data_as(ctypes.c_void_p), len(problems),
                                            _stream(stream)))


def batch_run_serial(problems: np.ndarray, stream=None) -> None:
    """Each problem by its own device-pointer call, in order (C loop)."""
    problems = np.ascontiguousarray(problems, dtype=PROBLEM_DTYPE)
    check(load().quadblas_batch_run_serial(problems.ctypes.data_as(ctypes.c_void_p), len(problems),
                                           _stream(stream)))


class BatchPlan:
    """A planned batch (quadblas_batch_plan); execute() replays it on a stream."""

    def __init__(self, problems: np.ndarray):
        problems = np.ascontiguousarray(problems, dtype=PROBLEM_DTYPE)
        self._problems = problems
        h = ctypes.c_void_p()
        check(load().quadblas_batch_plan(problems.ctypes.data_as(ctypes.c_void_p), len(problems),
                                         ctypes.byref(h)))
        self.handle = h

    def execute(self, stream=None) -> None:
        check(load().quadblas_batch_execute(self.handle, _stream(stream)))

    def info(self) -> dict:
        out = (ctypes.c_int64 * 7)()
        check(load().quadblas_batch_info_ex(self.handle, out, 7))
        return {"items": out[0], "grain": out[1], "blocks": out[2], "split_groups": out[3], "tile": out[4],
                "ozaki_problems": out[5], "ozaki_tiles": out[6]}

    def close(self) -> None:
        if self.handle:
            load().quadblas_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_autotune() -> int:
    g = ctypes.c_int64(0)
    check(load().quadblas_batch_autotune(ctypes.byref(g)))
    return g.value


def batch_set_grain(grain: int) -> None:
    check(load().quadblas_batch_set_grain(grain))


def batch_setting() -> tuple:
    """(granularity, gemm tile edge) that new plans on this device use."""
    g, t = ctypes.c_int64(0), ctypes.c_int(0)
    check(load().quadblas_batch_setting(ctypes.byref(g), ctypes.byref(t)))
    return g.value, t.value


def batch_configure(grain: int, tile: int = 0) -> None:
    check(load().quadblas_batch_configure(grain, tile))


def batch_set_ozaki_min(products: int) -> None:
    """Smallest m*n*k of a qgemm problem that new plans run on the grouped
    tensor-core path under the Ozaki method (0 = the default, 2^20)."""
    check(load().quadblas_batch_set_ozaki_min(products))
