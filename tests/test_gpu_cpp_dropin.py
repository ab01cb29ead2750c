"""The reference's C++ interface as a drop-in: tests/cpp_dropin.cpp uses
QuadBLAS::Vector / QuadBLAS::Matrix members exactly as a program written
for the reference would, is compiled against include/quadblas/quadblas.hpp
and linked to libquadblas_gpu.so, and runs on the GPU.  Its known answers are
checked inside the program; its results on random inputs are compared here
with the exact oracle (dot, gemv and gemm correctly rounded, axpy bit-exact
with fma, norm the correctly rounded square root of the correctly rounded
sum of squares), and the column-major gemm (B^T A^T) must reproduce the
row-major A B bit for bit."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from gpu_helpers import epilogue, rep
from qblas_gb300 import gen as G
from qblas_gb300 import quad as Q

pytestmark = pytest.mark.gpu


def test_cpp_dropin_program(qlib, O, tmp_path):
    libdir = os.path.join(ROOT, "qblas_gb300", "_build")
    exe = tmp_path / "cpp_dropin"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp_dropin.cpp"), "-L", libdir, "-lquadblas_gpu",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    n, m, k = 1000, 48, 40
    rng = G.rng_for(77)
    x, y = G.uniform_full(rng, n), G.wide_exponent(rng, n, -30, 30)
    A, B = G.uniform_full(rng, m * k), G.uniform_full(rng, k * m)
    v, w = G.uniform_full(rng, k), G.uniform_full(rng, m)
    inp, outp = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        f.write(np.array([n, m, k], dtype=np.int64).tobytes())
        for a in (x, y, A, B, v, w):
            f.write(np.ascontiguousarray(a).tobytes())
    subprocess.run([str(exe), str(inp), str(outp)], check=True)
    out = np.fromfile(outp, dtype=np.uint64).reshape(-1, 2)
    assert len(out) == 2 + n + m + k + 2 * m * m
    o = 0

    def take(cnt):
        nonlocal o
        o += cnt
        return out[o - cnt:o]

    R, _, _ = O.exact_dot(x, y)
    assert Q.same_bits(take(1), R).all()
    R2, _, _ = O.exact_dot(x, x)
    assert Q.same_bits(take(1), O.sqrt(R2)).all()
    assert Q.same_bits(take(n), O.fma(rep(Q.scalar(2.5), n), x, y)).all()
    Rg, _, _ = O.exact_gemv(m, k, A, k, 1, v)
    assert Q.same_bits(take(m), epilogue(O, Q.scalar(1.5), Rg, Q.scalar(0.5), w)).all()
    Rt, _, _ = O.exact_gemv(k, m, A, 1, k, w)
    assert Q.same_bits(take(k), Rt).all()
    rows, cols = np.meshgrid(np.arange(m), np.arange(m), indexing="ij")
    Rc, _, _ = O.exact_gemm(k, A, k, 1, B, m, 1, rows.ravel(), cols.ravel())
    C = take(m * m)
    assert Q.same_bits(C, Rc).all()
    assert Q.same_bits(take(m * m), C).all()
