"""GPU parity of the Ozaki qgemm, digit-pair scheme (tcgen05 digit products).

* Bit-exact against the CPU emulation of the same algorithm (ozaki_emul:
  the digit split and fold of ozaki.cuh built for the host, digit products
  as exact numpy int64 GEMMs): the tensor-core products are exact integers,
  so any difference is a defect of the GPU path.
* Accuracy against the exact oracle: with 17 digits of 8 bits (or 20 of 7
  bits) per operand the result is within 1 ulp (u_q = 2^-113) of the exact
  sum on spread-exponent data (e uniform in [-20, 20]).
* NaN / infinity rows and columns follow the exact-oracle semantics.
"""
import ctypes

import numpy as np
import pytest

import ozaki_emul as E
from conftest import to_dev, to_host
from gpu_helpers import epilogue
from qblas_gb300 import api
from qblas_gb300 import gen as G
from qblas_gb300 import quad as Q

pytestmark = pytest.mark.gpu


@pytest.fixture
def ozaki(qlib):
    api.set_method(2)
    api.set_ozaki_scheme(1)  # digit pairs (the residue scheme: test_gpu_ozcrt.py)
    yield qlib
    api.set_method(0)
    api.set_ozaki_scheme(0)
    api.set_ozaki_slices(0)
    api.set_ozaki_digit_bits(0)


def strides(layout, ta, tb, lda, ldb, ldc):
    col = layout == "C"
    if not col:
        sa = (1, lda) if ta else (lda, 1)
        sb = (1, ldb) if tb else (ldb, 1)
        sc = (ldc, 1)
    else:
        sa = (lda, 1) if ta else (1, lda)
        sb = (ldb, 1) if tb else (1, ldb)
        sc = (1, ldc)
    return sa, sb, sc


def run_case(O, sq, rng, layout, transa, transb, m, n, k, s, gen, al_d, be_d, b=8):
    col = layout == "C"
    ta, tb = transa == "T", transb == "T"
    ar, ac = (k, m) if ta else (m, k)
    br, bc = (n, k) if tb else (k, n)
    lda = (ar if col else ac) + 1
    ldb = (br if col else bc) + 2
    ldc = (m if col else n) + 1
    A = gen(rng, (ac if col else ar) * lda)
    B = gen(rng, (bc if col else br) * ldb)
    C = G.uniform_full(rng, (n if col else m) * ldc)
    alpha, beta = Q.scalar(al_d), Q.scalar(be_d)
    api.set_ozaki_slices(s)
    api.set_ozaki_digit_bits(b)
    got = C.copy()
    api.gemm(layout, transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, got, ldc)
    (sai, sal), (sbl, sbj), (sci, scj) = strides(layout, ta, tb, lda, ldb, ldc)
    sums = E.gemm_sum(sq, m, n, k, A, sai, sal, B, sbl, sbj, s, b)
    rows, cols = np.meshgrid(np.arange(m), np.arange(n), indexing="ij")
    idx = rows.ravel() * sci + cols.ravel() * scj
    exp = epilogue(O, alpha, sums, beta, C[idx])
    return got, idx, exp, (A, sai, sal, B, sbl, sbj)


def test_ozaki_one_tile_bit_exact(ozaki, O, sq):
    """Smallest case first: one 128 x 256 tile, one K block."""
    rng = G.rng_for(1)
    got, idx, exp, _ = run_case(O, sq, rng, "R", "N", "N", 128, 256, 64, 2, G.spread_uniform, 1.0, 0.0)
    assert Q.same_bits(got[idx], exp).all()


@pytest.mark.parametrize("s,b", [(2, 8), (7, 8), (18, 8), (20, 8), (7, 7), (20, 7), (2, 9), (15, 9), (18, 9)])
def test_ozaki_bit_exact_vs_emulation(ozaki, O, sq, s, b):
    rng = G.rng_for(10 + s + 100 * b)
    cases = [("R", "N", "N", 1, 1, 1), ("R", "N", "N", 5, 7, 9), ("R", "T", "N", 130, 257, 70),
             ("C", "N", "N", 200, 100, 300), ("C", "T", "T", 33, 290, 129), ("R", "N", "T", 129, 255, 65)]
    for layout, ta, tb, m, n, k in cases:
        got, idx, exp, _ = run_case(O, sq, rng, layout, ta, tb, m, n, k, s, G.spread_uniform, 2.5, -1.5, b)
        assert Q.same_bits(got[idx], exp).all(), (layout, ta, tb, m, n, k, s, b)


@pytest.mark.parametrize("b,k", [(7, 4096 + 64 + 5), (8, 3 * 1024 + 64 + 5), (9, 5 * 256 + 64 + 5)])
def test_ozaki_several_exact_chunks(ozaki, O, sq, b, k):
    """k above the fp32-exact chunk (4096 for 7-bit, 1024 for 8-bit, 256 for
    9-bit digits): chunk sums are read out of tensor memory and added in int32."""
    rng = G.rng_for(2 + b)
    got, idx, exp, _ = run_case(O, sq, rng, "R", "N", "N", 128, 256, k, 6, G.spread_uniform, 1.0, 0.0, b)
    assert Q.same_bits(got[idx], exp).all()


@pytest.mark.parametrize("s,b,k", [(15, 9, 2048 + 300), (18, 9, 1792 + 77), (17, 8, 7168 + 129), (20, 7, 6 * 4096 + 65)])
def test_ozaki_several_k_passes(ozaki, O, sq, s, b, k):
    """k above one pass (the int32 diagonal sums hold (2^31 - 1) / (s 2^24)
    exact chunks): each pass writes its own diagonal planes and the fold adds
    them; bit-exact with the emulation."""
    rng = G.rng_for(20 + s + b)
    for layout, ta, tb, m, n in (("R", "N", "N", 24, 40), ("C", "T", "N", 17, 33)):
        got, idx, exp, _ = run_case(O, sq, rng, layout, ta, tb, m, n, k, s, G.spread_uniform, 1.0, 0.5, b)
        assert Q.same_bits(got[idx], exp).all(), (layout, s, b, k)


def test_ozaki_mixed_magnitudes(ozaki, O, sq):
    """Zero rows, subnormal and huge entries go through the same split."""
    rng = G.rng_for(3)

    def gen(rng, n):
        q = G.wide_exponent(rng, n, -16000, 16000)
        q[: n // 7] = 0
        return q

    for b, s in ((8, 18), (7, 20), (9, 16)):
        got, idx, exp, _ = run_case(O, sq, rng, "R", "N", "N", 67, 301, 45, s, gen, 1.0, 0.0, b)
        assert Q.same_bits(got[idx], exp).all(), b


@pytest.mark.parametrize("size,s,b", [(512, 18, 8), (512, 20, 7), (4096, 17, 8), (4096, 15, 9)])
def test_ozaki_accuracy_spread(ozaki, O, torch_cuda, size, s, b):
    """size^3 on e-uniform-[-20, 20] data (the 4096^3 benchmark workload at
    its digit count): every sampled entry is within 1 ulp of the exact sum."""
    torch = torch_cuda
    m = n = k = size
    rng = G.rng_for(0xC0FFEE + 2)
    A, B = G.spread_uniform(rng, m * k), G.spread_uniform(rng, k * n)
    C = Q.from_double(np.zeros(m * n))
    dA, dB, dC = to_dev(torch, A), to_dev(torch, B), to_dev(torch, C)
    api.set_ozaki_slices(s)
    api.set_ozaki_digit_bits(b)
    api.gemm_dev("R", "N", "N", m, n, k, Q.scalar(1.0), dA, k, dB, n, Q.scalar(0.0), dC, n)
    torch.cuda.synchronize()
    got = to_host(dC)
    nsamp = 20000 if size <= 512 else 6000
    rows, cols = rng.integers(0, m, nsamp), rng.integers(0, n, nsamp)
    R, r, _ = O.exact_gemm(k, A, k, 1, B, n, 1, rows, cols, nthreads=16)
    err = O.ulp_err(got[rows * n + cols], R, r)
    assert err.max() <= 1.0, err.max()


def test_ozaki_special_values(ozaki, O):
    rng = G.rng_for(4)
    m, n, k = 9, 11, 13
    A, B = G.uniform_full(rng, m * k), G.uniform_full(rng, k * n)
    A[2 * k + 3] = [0, 0x7FFF800000000000]   # NaN in row 2
    A[5 * k + 1] = [0, 0x7FFF000000000000]   # +inf in row 5
    B[4 * n + 7] = [0, 0xFFFF000000000000]   # -inf in column 7
    C = Q.from_double(np.zeros(m * n))
    got = C.copy()
    api.gemm("R", "N", "N", m, n, k, Q.scalar(1.0), A, k, B, n, Q.scalar(0.0), got, n)
    rows, cols = np.meshgrid(np.arange(m), np.arange(n), indexing="ij")
    R, _, _ = O.exact_gemm(k, A, k, 1, B, n, 1, rows.ravel(), cols.ravel())
    special = np.zeros((m, n), bool)
    special[[2, 5], :] = True
    special[:, 7] = True
    sp = special.ravel()
    assert Q.same_bits(got[sp], R[sp]).all()
    # the other entries come from the digit products
    assert Q.is_nan(got[~sp]).sum() == 0


def test_ozaki_reference_c_interface(ozaki, O, sq):
    """quadblas_qgemm with the Ozaki method through host pointers."""
    rng = G.rng_for(5)
    m, n, k = 40, 50, 60
    A, B, C = G.spread_uniform(rng, m * k), G.spread_uniform(rng, k * n), G.uniform_full(rng, m * n)
    got = C.copy()
    api.qgemm("R", "N", "N", m, n, k, 2.0, A, k, B, n, 0.5, got, n)  # library defaults: 16 digits of 9 bits
    sums = E.gemm_sum(sq, m, n, k, A, k, 1, B, n, 1, 16, 9)
    assert Q.same_bits(got, epilogue(O, Q.scalar(2.0), sums, Q.scalar(0.5), C)).all()
