"""GPU parity of the Ozaki qgemm, residue (CRT) scheme: quadblas_set_ozaki_scheme(2).

* Bit-exact against the CPU emulation of the same algorithm
  (ozaki_emul.crt_gemm_sum: the residue split and reconstruction of
  ozcrt.cuh built for the host, residue products as exact numpy int64
  GEMMs).  The emulation itself equals the correctly rounded exact sum of the
  T-bit truncated products (tests/test_ozcrt_host.py), so the tolerance is
  none.
* Accuracy against the exact oracle: with T = 134 bits (15 slices of 9
  bits, the 4096^3 benchmark setting) every sampled entry is within 1 ulp
  (u_q = 2^-113) of the exact sum on spread-exponent data.
* NaN / infinity rows and columns follow the exact-oracle semantics.
"""
import numpy as np
import pytest

import ozaki_emul as E
from conftest import to_dev, to_host
from gpu_helpers import epilogue
from qblas_gb300 import api
from qblas_gb300 import gen as G
from qblas_gb300 import quad as Q
from test_gpu_ozaki import strides

pytestmark = pytest.mark.gpu


@pytest.fixture
def crt(qlib):
    api.set_method(2)
    api.set_ozaki_scheme(2)
    yield qlib
    api.set_method(0)
    api.set_ozaki_scheme(0)
    api.set_ozaki_slices(0)
    api.set_ozaki_digit_bits(0)


def run_case(O, sq, rng, layout, transa, transb, m, n, k, s, gen, al_d, be_d, b=9, torch=None, c_specials=False):
    """One call (host pointers, or device pointers when torch is given)
    against the emulation of the same algorithm; c_specials plants NaN,
    +-inf and +-0 in C (what beta * C makes of them is the epilogue's)."""
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
    if c_specials:
        specials = [[0, 0x7FFF800000000000], [0, 0x7FFF000000000000], [0, 0xFFFF000000000000],
                    [0, 0x8000000000000000], [0, 0]]
        for t, pos in enumerate(rng.choice(len(C), size=5 * 7, replace=False)):
            C[pos] = specials[t % 5]
    alpha, beta = Q.scalar(al_d), Q.scalar(be_d)
    api.set_ozaki_slices(s)
    api.set_ozaki_digit_bits(b)
    if torch is None:
        got = C.copy()
        api.gemm(layout, transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, got, ldc)
    else:
        dA, dB, dC = to_dev(torch, A), to_dev(torch, B), to_dev(torch, C)
        api.gemm_dev(layout, transa, transb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc)
        torch.cuda.synchronize()
        got = to_host(dC)
    (sai, sal), (sbl, sbj), (sci, scj) = strides(layout, ta, tb, lda, ldb, ldc)
    sums = E.crt_gemm_sum(sq, m, n, k, A, sai, sal, B, sbl, sbj, b * s - 1)
    rows, cols = np.meshgrid(np.arange(m), np.arange(n), indexing="ij")
    idx = rows.ravel() * sci + cols.ravel() * scj
    exp = epilogue(O, alpha, sums, beta, C[idx])
    return got, idx, exp


def test_crt_one_tile_bit_exact(crt, O, sq):
    """Smallest case first: one 128 x 256 tile, one K block."""
    rng = G.rng_for(401)
    got, idx, exp = run_case(O, sq, rng, "R", "N", "N", 128, 256, 64, 15, G.spread_uniform, 1.0, 0.0)
    assert Q.same_bits(got[idx], exp).all()


# T = b*s - 1: 71 and 103 (8-word reconstruction), 134 and 143 (10 words, 9
# pieces), 153 (12 pieces), 161 (12 pieces, 12 words)
@pytest.mark.parametrize("s,b", [(8, 9), (13, 8), (15, 9), (16, 9), (22, 7), (18, 9)])
def test_crt_bit_exact_vs_emulation(crt, O, sq, s, b):
    rng = G.rng_for(410 + s + 100 * b)
    cases = [("R", "N", "N", 1, 1, 1), ("R", "N", "N", 5, 7, 9), ("R", "T", "N", 130, 257, 70),
             ("C", "N", "N", 200, 100, 300), ("C", "T", "T", 33, 290, 129), ("R", "N", "T", 129, 255, 65)]
    for layout, ta, tb, m, n, k in cases:
        got, idx, exp = run_case(O, sq, rng, layout, ta, tb, m, n, k, s, G.spread_uniform, 2.5, -1.5, b)
        assert Q.same_bits(got[idx], exp).all(), (layout, ta, tb, m, n, k, s, b)


def test_crt_several_chunks_and_passes(crt, O, sq):
    """k above the fp32-exact chunk (256) and above one pass (8192: the int32
    residue sums stay within 2^29); each pass writes its own planes and the
    reconstruction adds their residues."""
    rng = G.rng_for(420)
    for layout, ta, tb, m, n, k in (("R", "N", "N", 128, 256, 5 * 256 + 69),
                                     ("R", "N", "N", 24, 40, 8192 + 300), ("C", "T", "N", 17, 33, 2 * 8192 + 65)):
        got, idx, exp = run_case(O, sq, rng, layout, ta, tb, m, n, k, 15, G.spread_uniform, 1.0, 0.5)
        assert Q.same_bits(got[idx], exp).all(), (layout, k)


def test_crt_mixed_magnitudes(crt, O, sq):
    """Zero rows, subnormal and huge entries go through the same split."""
    rng = G.rng_for(421)

    def gen(rng, n):
        q = G.wide_exponent(rng, n, -16000, 16000)
        q[: n // 7] = 0
        return q

    for b, s in ((9, 16), (8, 18), (7, 20)):
        got, idx, exp = run_case(O, sq, rng, "R", "N", "N", 67, 301, 45, s, gen, 1.0, 0.0, b)
        assert Q.same_bits(got[idx], exp).all(), b


@pytest.mark.parametrize("layout,transa,transb,m,n,k", [("R", "N", "N", 70, 90, 300), ("R", "T", "N", 65, 33, 129),
                                                     ("C", "N", "T", 129, 70, 65), ("C", "T", "T", 33, 290, 129),
                                                     ("R", "N", "T", 300, 257, 1000), ("R", "N", "N", 600, 130, 200),
                                                     ("R", "N", "N", 320, 400, 150), ("C", "T", "T", 300, 400, 90)])
def test_crt_device_pointer_bit_exact(crt, O, sq, torch_cuda, layout, transa, transb, m, n, k):
    """Device-pointer calls on one stream: op(A)'s scales come from the side
    warp of op(B)'s residue split where op(A)'s rows are contiguous and the
    side job ends within the split (300 m <= n min(m, split grid): the
    320 x 400 x 150 and 300 x 400 x 90 cases, and 300 x 257 x 1000), from
    their own launch otherwise (transposed layouts, small n, 600 > 2 * 130);
    bit-exact against the emulation either way."""
    rng = G.rng_for(431 + m)
    got, idx, exp = run_case(O, sq, rng, layout, transa, transb, m, n, k, 15, G.spread_uniform, 1.5, -0.75,
                             torch=torch_cuda)
    assert Q.same_bits(got[idx], exp).all(), int((~Q.same_bits(got[idx], exp)).sum())


@pytest.mark.parametrize("device", [False, True])
@pytest.mark.parametrize("al_d,be_d", [(1.0, 0.0), (1.0, -0.0), (2.0, 0.0), (-1.0, -0.0)])
def test_crt_beta_zero_with_special_c(crt, O, sq, request, device, al_d, be_d):
    """beta = +-0 with NaN, +-inf and +-0 already in C: every output is
    fma(alpha, sum, beta * C) as the reference epilogue forms it (NaN where
    C held NaN or inf, the sign of a zero sum from beta * C), with the
    epilogue's fast path for alpha = 1 and the product path otherwise."""
    torch = request.getfixturevalue("torch_cuda") if device else None
    rng = G.rng_for(451)
    got, idx, exp = run_case(O, sq, rng, "R", "N", "N", 37, 45, 70, 15, G.spread_uniform, al_d, be_d,
                             torch=torch, c_specials=True)
    assert Q.same_bits(got[idx], exp).all(), int((~Q.same_bits(got[idx], exp)).sum())


@pytest.mark.parametrize("size", [512, 4096])
def test_crt_accuracy_spread(crt, O, torch_cuda, size):
    """size^3 on e-uniform-[-20, 20] data at the benchmark setting (15 slices
    of 9 bits: T = 134): every sampled entry is within 1 ulp of the exact sum."""
    torch = torch_cuda
    m = n = k = size
    rng = G.rng_for(0xC0FFEE + 2)
    A, B = G.spread_uniform(rng, m * k), G.spread_uniform(rng, k * n)
    C = Q.from_double(np.zeros(m * n))
    dA, dB, dC = to_dev(torch, A), to_dev(torch, B), to_dev(torch, C)
    api.set_ozaki_slices(15)
    api.set_ozaki_digit_bits(9)
    api.gemm_dev("R", "N", "N", m, n, k, Q.scalar(1.0), dA, k, dB, n, Q.scalar(0.0), dC, n)
    torch.cuda.synchronize()
    got = to_host(dC)
    nsamp = 20000 if size <= 512 else 6000
    rows, cols = rng.integers(0, m, nsamp), rng.integers(0, n, nsamp)
    R, r, _ = O.exact_gemm(k, A, k, 1, B, n, 1, rows, cols, nthreads=16)
    err = O.ulp_err(got[rows * n + cols], R, r)
    assert err.max() <= 1.0, err.max()


@pytest.mark.parametrize("scheme", [2, 1])
@pytest.mark.parametrize("shape,pinned", [((1664, 3072, 96), False), ((4000, 2100, 70), True),
                                          ((4000, 2100, 70), False)])
def test_host_pointer_row_bands_match_device(crt, torch_cuda, scheme, shape, pinned):
    """A host-pointer qgemm with more 128 x 256 tiles than the GPU has SMs
    runs in row bands: A is copied band by band, and C is folded and copied
    back in row bands.  At 13 x 12 = 156 tiles the products are one band and
    the fold four.  At 32 x 9 = 288 tiles (m and n off the tile grid) the
    products are two bands; from page-locked buffers the same rows of C
    follow each band of A and the rows of the first band are folded before
    the second multiplies (the rest in one band), from pageable buffers C
    comes whole after A.  With beta != 0 and a random C the result must
    equal the device-pointer call's bit for bit; a fold that ran before its
    rows of C arrived would read the staging buffer's previous contents
    (another call's result, left there on purpose)."""
    torch = torch_cuda
    if pinned:
        keep = lambda a: torch.from_numpy(a.view(np.int64)).pin_memory().numpy().view(np.uint64)  # noqa: E731
    else:
        keep = lambda a: a  # noqa: E731
    api.set_ozaki_scheme(scheme)
    api.set_ozaki_slices(15)
    api.set_ozaki_digit_bits(9)
    m, n, k = shape
    rng = G.rng_for(424 + scheme)
    A, B, C = G.spread_uniform(rng, m * k), G.spread_uniform(rng, k * n), G.uniform_full(rng, m * n)
    alpha, beta = Q.scalar(1.25), Q.scalar(-0.75)
    dA, dB, dC = to_dev(torch, A), to_dev(torch, B), to_dev(torch, C)
    api.gemm_dev("R", "N", "N", m, n, k, alpha, dA, k, dB, n, beta, dC, n)
    torch.cuda.synchronize()
    ref = to_host(dC)
    A, B = keep(A), keep(B)
    other = keep(G.uniform_full(rng, m * n))
    api.gemm("R", "N", "N", m, n, k, alpha, A, k, B, n, Q.scalar(0.0), other, n)
    got = keep(C.copy())
    api.gemm("R", "N", "N", m, n, k, alpha, A, k, B, n, beta, got, n)
    assert Q.same_bits(got, ref).all(), int((~Q.same_bits(got, ref)).sum())


@pytest.mark.parametrize("device,m,n,k", [(False, 9, 11, 13), (True, 9, 11, 13), (True, 310, 320, 300)])
def test_crt_special_values(crt, O, device, m, n, k, request):
    """Host pointers, and device pointers on one stream (at 310 x 320 x 300
    op(A)'s row scales and flags come from the side warp of op(B)'s split)."""
    rng = G.rng_for(422)
    A, B = G.uniform_full(rng, m * k), G.uniform_full(rng, k * n)
    A[2 * k + 3] = [0, 0x7FFF800000000000]   # NaN in row 2
    A[5 * k + 1] = [0, 0x7FFF000000000000]   # +inf in row 5
    B[4 * n + 7] = [0, 0xFFFF000000000000]   # -inf in column 7
    C = Q.from_double(np.zeros(m * n))
    if device:
        torch = request.getfixturevalue("torch_cuda")
        dA, dB, dC = to_dev(torch, A), to_dev(torch, B), to_dev(torch, C)
        api.gemm_dev("R", "N", "N", m, n, k, Q.scalar(1.0), dA, k, dB, n, Q.scalar(0.0), dC, n)
        torch.cuda.synchronize()
        got = to_host(dC)
    else:
        got = C.copy()
        api.gemm("R", "N", "N", m, n, k, Q.scalar(1.0), A, k, B, n, Q.scalar(0.0), got, n)
    special = np.zeros((m, n), bool)
    special[[2, 5], :] = True
    special[:, 7] = True
    sp = special.ravel()
    rows, cols = np.nonzero(special)
    R, _, _ = O.exact_gemm(k, A, k, 1, B, n, 1, rows, cols)
    assert Q.same_bits(got[sp], R).all()
    assert Q.is_nan(got[~sp]).sum() == 0


def test_crt_default_scheme_and_c_interface(qlib, O, sq):
    """quadblas_qgemm with the Ozaki method and every setting at its default
    (automatic scheme: residues; 16 slices of 9 bits, T = 143)."""
    rng = G.rng_for(423)
    m, n, k = 40, 50, 60
    A, B, C = G.spread_uniform(rng, m * k), G.spread_uniform(rng, k * n), G.uniform_full(rng, m * n)
    api.set_method(2)
    try:
        assert api.get_ozaki_scheme() == 0
        got = C.copy()
        api.qgemm("R", "N", "N", m, n, k, 2.0, A, k, B, n, 0.5, got, n)
    finally:
        api.set_method(0)
    sums = E.crt_gemm_sum(sq, m, n, k, A, k, 1, B, n, 1, 16 * 9 - 1)
    assert Q.same_bits(got, epilogue(O, Q.scalar(2.0), sums, Q.scalar(0.5), C)).all()


@pytest.mark.parametrize("mode", [1, 2])
def test_profile_modes(crt, torch_cuda, mode):
    """quadblas_profile_enable: mode 1 times every phase of a device-pointer
    call, mode 2 only the tensor-core products (the other phases read 0)."""
    import ctypes
    from qblas_gb300._lib import load
    torch = torch_cuda
    lib = load()
    m = n = k = 256
    rng = G.rng_for(77)
    A, B = G.spread_uniform(rng, m * k), G.spread_uniform(rng, k * n)
    dA, dB, dC = to_dev(torch, A), to_dev(torch, B), to_dev(torch, Q.from_double(np.zeros(m * n)))
    out, calls = (ctypes.c_double * 4)(), ctypes.c_int(0)
    lib.quadblas_profile_read(out, ctypes.byref(calls))  # drop anything recorded before
    lib.quadblas_profile_enable(mode)
    try:
        for _ in range(3):
            api.gemm_dev("R", "N", "N", m, n, k, Q.scalar(1.0), dA, k, dB, n, Q.scalar(0.0), dC, n)
        torch.cuda.synchronize()
    finally:
        lib.quadblas_profile_enable(0)
    assert lib.quadblas_profile_read(out, ctypes.byref(calls)) == 0
    assert calls.value == 3
    products = out[3] / (3 * 2.0 * m * n * k)  # residue products per call (one per modulus)
    assert out[1] > 0 and 20 <= round(products) <= 48 and abs(products - round(products)) < 1e-3
    if mode == 1:
        assert out[0] > 0 and out[2] > 0
    else:
        assert out[0] == 0 and out[2] == 0


@pytest.mark.parametrize("k", [4096, 7600])
@pytest.mark.parametrize("sign", [1, -1])
def test_crt_largest_sums(crt, torch_cuda, k, sign):
    """Every operand 1 - 2^-113 and every product of one sign, T = 134: the
    largest sum the truncated operands allow, at 0.265 M (k = 4096) and
    0.4917 M (k = 7600, 32 moduli still) against the 32/65 M the
    reconstruction's quotient estimate is proved for; every output is the
    correctly rounded k (1 - 2^-113)^2."""
    from fractions import Fraction
    from test_oracle import fraction_to_q
    torch = torch_cuda
    m, n = 130, 70
    top = np.array([0xFFFFFFFFFFFFFFFF, 0x3FFEFFFFFFFFFFFF], dtype=np.uint64)
    A = np.tile(top, (m * k, 1))
    B = np.tile(top, (k * n, 1))
    if sign < 0:
        B[:, 1] |= np.uint64(1 << 63)
    dA, dB, dC = to_dev(torch, A), to_dev(torch, B), to_dev(torch, Q.from_double(np.zeros(m * n)))
    api.set_ozaki_slices(15)
    api.set_ozaki_digit_bits(9)
    api.gemm_dev("R", "N", "N", m, n, k, Q.scalar(1.0), dA, k, dB, n, Q.scalar(0.0), dC, n)
    torch.cuda.synchronize()
    got = to_host(dC)
    want = fraction_to_q(sign * k * (1 - Fraction(1, 1 << 113)) ** 2)
    assert (got[:, 0] == np.uint64(want[0])).all() and (got[:, 1] == np.uint64(want[1])).all()
