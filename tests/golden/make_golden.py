"""Generates tests/golden/reference_outputs.npz: seeded binary128 inputs
and the outputs of the reference QuadBLAS itself on them.

The reference is compiled from its own headers through the SLEEF shim
(oracle/_ref/libqref.so, built by `make -C oracle` where the reference
tree exists).  The fixtures let the oracle restatement be pinned against the
reference on machines that do not have the reference tree (the GPU machine):
tests/test_oracle.py checks that the restatement reproduces every output
bit for bit.

Cases mirror the reference's own tests (test_quadblas.cpp): the dot tests
(:205-260, with the OpenMP-parallel path, n >= 500, and a strided call),
axpy (:263-287), row- and column-major gemv with alpha=1.5, beta=0.5
(:353-370), the simple (<= 64) and blocked (> 64, several k-panels) gemm
paths with alpha=2.5, beta=1.5 (:573-590), and the known-answer inputs.

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from qblas_gb300 import gen as G  # noqa: E402
from qblas_gb300 import quad as Q  # noqa: E402

c64 = ctypes.c_int64
cint = ctypes.c_int


def main() -> None:
    O.build()
    R = O.ref_lib()
    if R is None:
        raise SystemExit("oracle/_ref/libqref.so is not built (reference tree absent)")
    P = O.P
    rng = G.rng_for(20251203)
    out = {}

    # --- dot: parallel contiguous path (T = 4), small path, strided path
    for name, n, incx, incy, T in [("dot_small", 10, 1, 1, 4), ("dot_par", 4099, 1, 1, 4),
                                   ("dot_strided", 600, 3, 2, 4), ("dot_strided_small", 77, 2, 3, 4)]:
        x = G.uniform_full(rng, n * incx)
        y = G.uniform_full(rng, n * incy)
        r = O.qs(1)
        R.qref_dot(c64(n), P(x), c64(incx), P(y), c64(incy), cint(T), P(r))
        out[f"{name}_x"], out[f"{name}_y"], out[f"{name}_out"] = x, y, r
        out[f"{name}_meta"] = np.array([n, incx, incy, T], dtype=np.int64)

    # --- axpy (alpha = 2.5)
    n = 1000
    x, y = G.uniform_full(rng, n), G.uniform_full(rng, n)
    al = Q.scalar(2.5)
    yr = y.copy()
    R.qref_axpy(c64(n), P(al), P(x), c64(1), P(yr), c64(1), cint(4))
    out["axpy_x"], out["axpy_y"], out["axpy_out"] = x, y, yr

    # --- gemv: row- and column-major, alpha = 1.5, beta = 0.5, library order
    for cm in (0, 1):
        m, n = 64, 80
        lda = n if cm == 0 else m
        A = G.uniform_full(rng, m * n)
        x, y = G.uniform_full(rng, n), G.uniform_full(rng, m)
        al, be = Q.scalar(1.5), Q.scalar(0.5)
        yr = y.copy()
        R.qref_gemv(cint(cm), c64(m), c64(n), P(al), P(A), c64(lda), P(x), c64(1), P(be), P(yr), c64(1),
                    cint(4))
        tag = f"gemv_{'col' if cm else 'row'}"
        out[f"{tag}_A"], out[f"{tag}_x"], out[f"{tag}_y"], out[f"{tag}_out"] = A, x, y, yr
        out[f"{tag}_meta"] = np.array([cm, m, n, lda], dtype=np.int64)

    # --- gemm row-major: simple path (16^3) and blocked path (k = 130 -> panels 126 + 4)
    for tag, (m, n, k) in [("gemm_simple", (16, 16, 16)), ("gemm_blocked", (70, 40, 130))]:
        A, B, C = G.uniform_full(rng, m * k), G.uniform_full(rng, k * n), G.uniform_full(rng, m * n)
        al, be = Q.scalar(2.5), Q.scalar(1.5)
        Cr = C.copy()
        R.qref_gemm(cint(0), c64(m), c64(n), c64(k), P(al), P(A), c64(k), P(B), c64(n), P(be), P(Cr), c64(n),
                    cint(4))
        out[f"{tag}_A"], out[f"{tag}_B"], out[f"{tag}_C"], out[f"{tag}_out"] = A, B, C, Cr
        out[f"{tag}_meta"] = np.array([m, n, k], dtype=np.int64)

    # --- known answers through the reference's C interface (double returns)
    kat = {}
    xs = Q.from_double(np.arange(1, 11, dtype=np.float64))
    ones = Q.from_double(np.ones(10))
    kat["dot_1_to_10"] = R.qref_c_qdot(cint(10), P(xs), cint(1), P(ones), cint(1))
    v = Q.from_double([1e20, 1.0, -1e20])
    w = Q.from_double([1.0, 1.0, 1.0])
    kat["dot_1e20_cancel"] = R.qref_c_qdot(cint(3), P(v), cint(1), P(w), cint(1))
    xs = Q.from_double(np.arange(1, 1001, dtype=np.float64))
    kat["nrm2_1_to_1000"] = R.qref_c_qnrm2(cint(1000), P(xs), cint(1))
    out["kat_names"] = np.array(list(kat.keys()))
    out["kat_values"] = np.array(list(kat.values()), dtype=np.float64)

    path = os.path.join(HERE, "reference_outputs.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path)} bytes)")


if __name__ == "__main__":
    main()
