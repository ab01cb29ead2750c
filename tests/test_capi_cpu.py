"""CPU-only checks of the C ABI library: it builds for sm_103a, exports
every symbol declared in include/quadblas_gpu.h, validates arguments on
the host, and fails loudly (no CPU fallback) when there is no GPU."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from qblas_gb300 import quad as Q

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HDR = os.path.join(ROOT, "include", "quadblas_gpu.h")


def declared_symbols():
    text = open(HDR).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(quadblas_\w+)\s*\(", text)))


def test_exports_every_declared_symbol(qlib):
    from qblas_gb300 import _lib
    syms = declared_symbols()
    assert len(syms) >= 25
    for s in syms:
        assert hasattr(qlib, s), s
    assert set(syms) == set(_lib.SYMBOLS)
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\b(quadblas_\w+)\b", out))
    assert set(syms) <= exported


def test_utilities(qlib):
    assert qlib.quadblas_get_version().startswith(b"QuadBLAS 1.0.0")
    buf = (ctypes.c_char * 128)()
    base = ctypes.addressof(buf)
    off = (-base) % 32
    assert qlib.quadblas_is_aligned(ctypes.c_void_p(base + off)) == 1
    assert qlib.quadblas_is_aligned(ctypes.c_void_p(base + off + 16)) == 0
    qlib.quadblas_set_num_threads(7)
    assert qlib.quadblas_get_num_threads() == 7
    assert qlib.quadblas_set_method(2) == 0 and qlib.quadblas_get_method() == 2
    assert qlib.quadblas_set_method(9) == 1
    qlib.quadblas_set_method(0)
    assert qlib.quadblas_set_ozaki_slices(12) == 0 and qlib.quadblas_get_ozaki_slices() == 12
    qlib.quadblas_set_ozaki_slices(0)
    assert qlib.quadblas_error_string(6) == b"device pointer not 16-byte aligned"
    assert qlib.quadblas_error_string(7).startswith(b"a device-side wait timed out")


def test_argument_validation_on_host(qlib):
    x = Q.from_double(np.ones(8))
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    res = Q.empty(1)
    assert qlib.quadblas_qdot_q(-1, P(x), 1, P(x), 1, P(res)) == 1
    assert qlib.quadblas_qdot_q(4, P(x), 0, P(x), 1, P(res)) == 1
    a = Q.scalar(1.0)
    # lda < k for row-major A (m x k)
    assert qlib.quadblas_qgemm_q(b"R", b"N", b"N", 2, 2, 4, P(a), P(x), 3, P(x), 2, P(a), P(x), 2) == 1
    # ldc < m for column-major C
    assert qlib.quadblas_qgemm_q(b"C", b"N", b"N", 4, 2, 2, P(a), P(x), 4, P(x), 2, P(a), P(x), 3) == 1
    # gemv: column-major needs lda >= m
    assert qlib.quadblas_qgemv_q(b"C", b"N", 4, 2, P(a), P(x), 3, P(x), 1, P(a), P(x), 1) == 1
    # transposed row-major A (stored m x n, read as its transpose): lda >= n
    assert qlib.quadblas_qgemv_q(b"R", b"T", 4, 3, P(a), P(x), 2, P(x), 1, P(a), P(x), 1) == 1
    assert qlib.quadblas_last_error() == 1
    # empty problems are no-ops (level2.hpp:21, level3.hpp:221)
    assert qlib.quadblas_qgemm_q(b"R", b"N", b"N", 0, 2, 2, P(a), P(x), 2, P(x), 2, P(a), P(x), 2) == 0
    assert qlib.quadblas_qaxpy_q(0, P(a), P(x), 1, P(x), 1) == 0


def test_no_cpu_fallback_without_gpu(qlib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    x = Q.from_double(np.arange(1, 11))
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    res = Q.empty(1)
    rc = qlib.quadblas_qdot_q(10, P(x), 1, P(x), 1, P(res))
    assert rc in (2, 5)  # CUDA error / no device: the call fails instead of computing on the CPU
    assert qlib.quadblas_qdot(10, P(x), 1, P(x), 1) == 0.0
    assert qlib.quadblas_last_error() in (2, 5)
    assert qlib.quadblas_device_status(1) in (2, 5)
    # the serial batch runner fails the same way (and checks its arguments first)
    assert qlib.quadblas_batch_run_serial(None, -1, None) == 1
    # batched controls: argument checks, then no device
    assert qlib.quadblas_batch_set_ozaki_min(-1) == 1
    assert qlib.quadblas_batch_set_ozaki_min(0) == 0
    assert qlib.quadblas_batch_configure(1 << 16, 24) == 1  # tile edge 16 or 32 only
    assert qlib.quadblas_qgemm_batched_dev(None, 0, None) in (2, 5)


def test_cpp_header_compiles(tmp_path):
    src = tmp_path / "t.cpp"
    src.write_text(
        '#include "quadblas/quadblas.hpp"\n'
        "int main() {\n"
        "  QuadBLAS::DefaultMatrix<> A(3, 3); QuadBLAS::DefaultVector<> x(3), y(3);\n"
        "  QuadBLAS::MatrixColMajor B(2, 2);\n"
        "  (void)A; (void)x; (void)y; (void)B; return 0; }\n")
    subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), str(src)],
                   check=True)
