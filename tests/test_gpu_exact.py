"""GPU parity of the certified soft-float path at any condition number.

Every soft-float result is the correctly rounded exact sum: the wide
accumulator's rounding is certified against its truncation budget, and the
outputs that cannot be certified (sums cancelling below the 256-bit frame)
are recomputed by the exact Kulisch fallback.  Checked bit for bit against
the exact oracle on GenDot sums of condition 1e40 to 1e60, a sum cancelling
across the whole exponent range, an exact rounding tie and an exact zero:
qdot (host, device, no-alloc and strided), qnrm2, qgemv (rows and columns
contiguous, with the reference epilogue), soft-float qgemm, and the batched
launch."""
import ctypes

import numpy as np
import pytest

from conftest import to_dev, to_host
from gpu_helpers import epilogue, rep
from qblas_gb300 import api
from qblas_gb300 import gen as G
from qblas_gb300 import quad as Q
from test_gpu_batched import Arena, check_all

pytestmark = pytest.mark.gpu


def hard_dots(O):
    """(name, x, y) pairs whose sums the 256-bit frame cannot round alone."""
    for cond, seed in ((1e40, 1), (1e50, 2), (1e60, 3), (1e30, 4)):
        x, y = O.gendot(8192, cond, seed)
        yield f"gendot {cond:.0e}", x, y
    big = Q.as_quad(Q.scalar(1.0)).copy()
    big[0, 1] = (np.uint64(16383 + 16000) << np.uint64(48)) | np.uint64(12345)
    negbig = big.copy()
    negbig[0, 1] ^= np.uint64(1 << 63)
    x = np.concatenate([big, Q.scalar(3.0), negbig, Q.scalar(2.0 ** -9000)])
    yield "full range", x, Q.from_double([1.0, 1.0, 1.0, 1.0])
    yield "tie", np.concatenate([Q.scalar(1.0), Q.scalar(2.0 ** -113)]), Q.from_double([1.0, 1.0])
    rng = G.rng_for(91)
    a = G.wide_exponent(rng, 1000, -3000, 3000)
    an = a.copy()
    an[:, 1] ^= np.uint64(1 << 63)
    b = G.wide_exponent(rng, 1000, -3000, 3000)
    yield "exact zero", np.concatenate([a, an]), np.concatenate([b, b])


def _dev_dot(fn, torch, n, dx, dy, incx=1, incy=1):
    out = torch.zeros((1, 2), dtype=torch.int64, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert fn(n, ctypes.c_void_p(dx.data_ptr()), incx, ctypes.c_void_p(dy.data_ptr()), incy,
              ctypes.c_void_p(out.data_ptr()), stream) == 0
    torch.cuda.synchronize()
    return to_host(out)


def test_qdot_any_condition(qlib, O, torch_cuda):
    torch = torch_cuda
    for name, x, y in hard_dots(O):
        R, _, _ = O.exact_dot(x, y)
        assert Q.same_bits(api.dot(x, y), R).all(), name
        dx, dy = to_dev(torch, x), to_dev(torch, y)
        assert Q.same_bits(_dev_dot(qlib.quadblas_qdot_dev, torch, len(x), dx, dy), R).all(), name
        assert Q.same_bits(_dev_dot(qlib.quadblas_qdot_dev_noalloc, torch, len(x), dx, dy), R).all(), name
        # strided: every other element
        xs, ys = np.repeat(x, 2, axis=0), np.repeat(y, 3, axis=0)
        assert Q.same_bits(api.dot(xs, ys, len(x), 2, 3), R).all(), name


def test_qnrm2_wide_range(qlib, O):
    rng = G.rng_for(92)
    x = G.wide_exponent(rng, 5000, -8000, 8000)
    R, _, _ = O.exact_dot(x, x)
    assert Q.same_bits(api.nrm2(x), O.sqrt(R)).all()


@pytest.mark.parametrize("layout,m", [("R", 40), ("C", 40), ("R", 4200)])
def test_qgemv_any_condition(qlib, O, layout, m):
    n = 4096
    x, y = O.gendot(n, 1e45, 8)
    rng = G.rng_for(93)
    rows = []
    for i in range(m):
        if i % 3 == 2:
            rows.append(G.uniform_full(rng, n))
        else:
            r = x.copy()  # exact power-of-two scaling keeps the condition
            r[:, 1] = r[:, 1] + (np.uint64(i % 7) << np.uint64(48))
            rows.append(r)
    Arows = np.stack(rows)  # m x n
    A = Arows.reshape(-1, 2) if layout == "R" else np.ascontiguousarray(Arows.transpose(1, 0, 2)).reshape(-1, 2)
    lda = n if layout == "R" else m
    yold = G.uniform_full(rng, m)
    alpha, beta = Q.scalar(1.5), Q.scalar(0.5)
    got = yold.copy()
    api.gemv(layout, "N", m, n, alpha, A, lda, y, 1, beta, got, 1)
    R, _, _ = O.exact_gemv(m, n, Arows.reshape(-1, 2), n, 1, y)
    assert Q.same_bits(got, epilogue(O, alpha, R, beta, yold)).all()


def test_qgemm_softfloat_any_condition(qlib, O):
    m = n = 48
    k = 2048
    conds = [1e40, 1e50, 1e60, 1e20] * (m // 4)
    X, Y = O.gendot_batch(k, conds, np.arange(m, dtype=np.uint64) + 77)
    A = X  # m x k row-major
    B = np.ascontiguousarray(Y.reshape(n, k, 2).transpose(1, 0, 2)).reshape(-1, 2)  # k x n, B[:, j] = y^(j)
    rng = G.rng_for(94)
    C0 = G.uniform_full(rng, m * n)
    alpha, beta = Q.scalar(1.0), Q.scalar(-0.5)
    got = C0.copy()
    api.set_method(0)
    api.gemm("R", "N", "N", m, n, k, alpha, A, k, B, n, beta, got, n)
    rows, cols = np.meshgrid(np.arange(m), np.arange(n), indexing="ij")
    R, _, _ = O.exact_gemm(k, A, k, 1, B, n, 1, rows.ravel(), cols.ravel())
    assert Q.same_bits(got, epilogue(O, alpha, R, beta, C0)).all()


@pytest.mark.parametrize("layout,ta,tb", [("C", "N", "N"), ("R", "T", "T"), ("C", "T", "N")])
def test_qgemm_softfloat_any_condition_layouts(qlib, O, layout, ta, tb):
    """The in-tile exact recomputation with every stride pattern of op(A), op(B), C."""
    m = n = 24
    k = 1536
    X, Y = O.gendot_batch(k, [1e45, 1e55, 1e20] * (m // 3), np.arange(m, dtype=np.uint64) + 300)
    Xr = X.reshape(m, k, 2)                       # op(A)(i, :) = x^(i)
    Yr = Y.reshape(n, k, 2)                       # op(B)(:, j) = y^(j)
    col = layout == "C"
    # store op(A) (m x k) and op(B) (k x n) in the requested layout and transposition
    opA = Xr
    opB = np.ascontiguousarray(Yr.transpose(1, 0, 2))
    stA = opA.transpose(1, 0, 2) if ta == "T" else opA   # the stored matrix before layout
    stB = opB.transpose(1, 0, 2) if tb == "T" else opB
    if col:
        stA, stB = stA.transpose(1, 0, 2), stB.transpose(1, 0, 2)
    A = np.ascontiguousarray(stA).reshape(-1, 2)
    B = np.ascontiguousarray(stB).reshape(-1, 2)
    lda, ldb = stA.shape[1], stB.shape[1]
    C0 = G.uniform_full(G.rng_for(97), m * n)
    got = C0.copy()
    api.set_method(0)
    api.gemm(layout, ta, tb, m, n, k, Q.scalar(1.0), A, lda, B, ldb, Q.scalar(0.25), got, n if not col else m)
    rows, cols = np.meshgrid(np.arange(m), np.arange(n), indexing="ij")
    R, _, _ = O.exact_gemm(k, Xr.reshape(-1, 2), k, 1, np.ascontiguousarray(opB).reshape(-1, 2), n, 1,
                           rows.ravel(), cols.ravel())
    idx = rows.ravel() * n + cols.ravel() if not col else cols.ravel() * m + rows.ravel()
    assert Q.same_bits(got[idx], epilogue(O, Q.scalar(1.0), R, Q.scalar(0.25), C0[idx])).all()


def test_batched_any_condition(qlib, O, torch_cuda):
    torch = torch_cuda
    ar = Arena(torch)
    specs = []
    for name, x, y in hard_dots(O):
        r = Q.from_double([7.0])
        specs.append(dict(op=2, layout="R", ta="N", tb="N", m=0, n=len(x), k=0, al=1.0, be=0.0, A=x, B=y, C=r,
                          lda=1, ldb=1, ldc=1, oA=ar.add(x), oB=ar.add(y), oC=ar.add(r)))
    k = 1024
    X, Y = O.gendot_batch(k, [1e40] * 8, np.arange(8, dtype=np.uint64) + 5)
    B = np.ascontiguousarray(Y.reshape(8, k, 2).transpose(1, 0, 2)).reshape(-1, 2)
    C = G.uniform_full(G.rng_for(95), 64)
    specs.append(dict(op=0, layout="R", ta="N", tb="N", m=8, n=8, k=k, al=2.0, be=0.5, A=X, B=B, C=C,
                      lda=k, ldb=8, ldc=8, oA=ar.add(X), oB=ar.add(B), oC=ar.add(C)))
    yv = G.uniform_full(G.rng_for(96), 8)
    specs.append(dict(op=1, layout="R", ta="N", tb="N", m=8, n=k, k=0, al=1.0, be=0.25, A=X,
                      B=Y[:k].copy(), C=yv, lda=k, ldb=1, ldc=1, oA=ar.add(X), oB=ar.add(Y[:k].copy()),
                      oC=ar.add(yv)))
    ar.upload()
    probs = np.zeros(len(specs), dtype=api.PROBLEM_DTYPE)
    for p, s in zip(probs, specs):
        p["op"] = s["op"]
        p["layout"], p["transa"], p["transb"] = s["layout"].encode(), s["ta"].encode(), s["tb"].encode()
        p["m"], p["n"], p["k"] = s["m"], s["n"], s["k"]
        p["alpha"], p["beta"] = Q.scalar(s["al"])[0], Q.scalar(s["be"])[0]
        p["A"], p["B"], p["C"] = ar.ptr(s["oA"]), ar.ptr(s["oB"]), ar.ptr(s["oC"])
        p["lda"], p["ldb"], p["ldc"] = s["lda"], s["ldb"], s["ldc"]
    for grain in (1024, 1 << 16):  # split and unsplit items
        ar.dev.copy_(to_dev(torch, ar.all))
        api.batch_set_grain(grain)
        plan = api.BatchPlan(probs)
        plan.execute()
        torch.cuda.synchronize()
        check_all(O, ar, specs)
        plan.close()
