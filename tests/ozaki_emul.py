"""CPU emulation of the Ozaki qgemm pipeline for the parity tests.

The digit split and the fold are the device code itself (ozaki.cuh) built
for the host (tests/softquad_host.cpp); the digit products are exact
numpy int64 matrix products.  Given the same inputs and digit count, the GPU
path must reproduce this emulation bit for bit: the tensor-core products
are exact integers, so any difference is a defect."""
import ctypes

import numpy as np

P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
c64 = ctypes.c_int64


def split(sq, X, rows, cols, sr, sc, s, b=8):
    S = np.zeros(rows, dtype=np.int32)
    D = np.zeros((s, rows, cols), dtype=np.int32)
    sq.sq_ozaki_split(c64(rows), c64(cols), P(np.ascontiguousarray(X)), c64(sr), c64(sc), ctypes.c_int(s),
                      ctypes.c_int(b), P(S), P(D))
    return S, D


def diagonals(DA, DB):
    """C_g = sum_{t+u=g, g<=s-1} DA_t @ DB_u^T (int64, exact)."""
    s = DA.shape[0]
    A64, B64 = DA.astype(np.int64), DB.astype(np.int64)
    C = np.zeros((s, DA.shape[1], DB.shape[1]), dtype=np.int64)
    for g in range(s):
        for t in range(g + 1):
            C[g] += A64[t] @ B64[g - t].T
    return C


def fold(sq, C, S, F, b=8):
    G = C.shape[0] - 1
    m, n = C.shape[1], C.shape[2]
    out = np.zeros((m * n, 2), dtype=np.uint64)
    sq.sq_ozaki_fold(c64(m), c64(n), ctypes.c_int(G), ctypes.c_int(b), P(np.ascontiguousarray(C)), P(S), P(F),
                     P(out))
    return out


def gemm_sum(sq, m, n, k, A, sai, sal, B, sbl, sbj, s, b=8):
    """round(sum_l op(A)(i,l) op(B)(l,j)) as the Ozaki path computes it with
    s digits of b bits, row-major (m*n, 2)."""
    SA, DA = split(sq, A, m, k, sai, sal, s, b)
    SB, DB = split(sq, B, n, k, sbj, sbl, s, b)  # op(B)^T rows = columns of op(B)
    return fold(sq, diagonals(DA, DB), SA, SB, b)


def crt_split(sq, X, rows, cols, sr, sc, T, k):
    """Row scales and the balanced residues R[q][r][c] of the CRT scheme."""
    nmax = 48
    S = np.zeros(rows, dtype=np.int32)
    R = np.zeros((nmax, rows, cols), dtype=np.int32)
    n = sq.sq_crt_split(c64(rows), c64(cols), P(np.ascontiguousarray(X)), c64(sr), c64(sc), ctypes.c_int(T),
                        c64(k), P(S), P(R))
    assert n > 0
    return S, R[:n]


def crt_gemm_sum(sq, m, n, k, A, sai, sal, B, sbl, sbj, T):
    """round(sum_l op(A)(i,l) op(B)(l,j)) as the CRT scheme computes it for
    T-bit operands: host residues, exact int64 residue products per modulus,
    host reconstruction; row-major (m*n, 2)."""
    SA, RA = crt_split(sq, A, m, k, sai, sal, T, k)
    SB, RB = crt_split(sq, B, n, k, sbj, sbl, T, k)
    C = np.stack([RA[q].astype(np.int64) @ RB[q].astype(np.int64).T for q in range(RA.shape[0])])
    out = np.zeros((m * n, 2), dtype=np.uint64)
    assert sq.sq_crt_fold(c64(m), c64(n), ctypes.c_int(T), c64(k), P(np.ascontiguousarray(C)), P(SA), P(SB),
                          P(out)) > 0
    return out
