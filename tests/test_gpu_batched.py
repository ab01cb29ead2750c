"""GPU parity of the batched persistent launch (quadblas_batch_*).

Every problem of a mixed batch (qgemm in both layouts and all transpose
combinations, qgemv row/column-major and transposed with strides, qdot with
strides and n = 0) must equal the single-call semantics bit for bit:
y = fma(alpha, R, beta*y) with R the correctly rounded exact sum (exact
long accumulator), qdot = R.  A small work-item granularity forces split-k
gemm tiles, column-split gemv rows and chunked dots, so the in-order merge
of partials is exercised; a re-execution, a CUDA-graph replay and the
autotuner are checked too."""

import numpy as np
import pytest

from conftest import to_dev, to_host
from gpu_helpers import epilogue
from qblas_gb300 import api
from qblas_gb300 import gen as G
from qblas_gb300 import quad as Q

pytestmark = pytest.mark.gpu


class Arena:
    """One device buffer holding every operand, carved into 16-byte elements."""

    def __init__(self, torch):
        self.torch, self.host = torch, []
        self.n = 0

    def add(self, q):
        off = self.n
        self.host.append(q)
        self.n += len(q)
        return off

    def upload(self):
        self.all = np.concatenate(self.host) if self.host else np.zeros((0, 2), np.uint64)
        self.dev = to_dev(self.torch, self.all)
        self.base = self.dev.data_ptr()

    def ptr(self, off):
        return self.base + 16 * off

    def read(self):
        return to_host(self.dev)


def make_batch(torch, rng, ngemm, ngemv, ndot):
    ar = Arena(torch)
    specs = []
    for _ in range(ngemm):
        m, n, k = (int(v) for v in rng.integers(1, 70, 3))
        layout = "RC"[rng.integers(2)]
        ta, tb = "NT"[rng.integers(2)], "NT"[rng.integers(2)]
        col = layout == "C"
        a_r, a_c = (k, m) if ta == "T" else (m, k)
        b_r, b_c = (n, k) if tb == "T" else (k, n)
        lda = (a_r if col else a_c) + int(rng.integers(0, 3))
        ldb = (b_r if col else b_c) + int(rng.integers(0, 3))
        ldc = (m if col else n) + int(rng.integers(0, 3))
        A = G.uniform_full(rng, (a_c if col else a_r) * lda)
        B = G.uniform_full(rng, (b_c if col else b_r) * ldb)
        C = G.uniform_full(rng, (n if col else m) * ldc)
        al, be = [(1.0, 0.0), (2.5, -1.5), (-0.75, 2.0)][rng.integers(3)]
        specs.append(dict(op=0, layout=layout, ta=ta, tb=tb, m=m, n=n, k=k, al=al, be=be, A=A, B=B, C=C,
                          lda=lda, ldb=ldb, ldc=ldc, oA=ar.add(A), oB=ar.add(B), oC=ar.add(C)))
    for _ in range(ngemv):
        m, n = (int(v) for v in rng.integers(1, 700, 2))
        layout, tr = "RC"[rng.integers(2)], "NT"[rng.integers(2)]
        incx, incy = int(rng.integers(1, 3)), int(rng.integers(1, 3))
        col = layout == "C"
        lda = (m if col else n) + int(rng.integers(0, 3))
        A = G.uniform_full(rng, (n if col else m) * lda)
        xl, yl = (m, n) if tr == "T" else (n, m)
        x, y = G.uniform_full(rng, xl * incx), G.uniform_full(rng, yl * incy)
        al, be = [(1.0, 0.0), (1.5, 0.5)][rng.integers(2)]
        specs.append(dict(op=1, layout=layout, ta=tr, tb="N", m=m, n=n, k=0, al=al, be=be, A=A, B=x, C=y,
                          lda=lda, ldb=incx, ldc=incy, oA=ar.add(A), oB=ar.add(x), oC=ar.add(y)))
    for i in range(ndot):
        n = 0 if i == 0 else int(rng.integers(1, 6000))
        incx, incy = int(rng.integers(1, 3)), int(rng.integers(1, 3))
        x, y = G.cancelling_dot(rng, max(n * max(incx, incy), 4))
        x, y = x[: max(n * incx, 1)], y[: max(n * incy, 1)]
        r = Q.from_double([7.0])
        specs.append(dict(op=2, layout="R", ta="N", tb="N", m=0, n=n, k=0, al=1.0, be=0.0, A=x, B=y, C=r,
                          lda=incx, ldb=incy, ldc=1, oA=ar.add(x), oB=ar.add(y), oC=ar.add(r)))
    ar.upload()
    probs = np.zeros(len(specs), dtype=api.PROBLEM_DTYPE)
    for p, s in zip(probs, specs):
        p["op"] = s["op"]
        p["layout"], p["transa"], p["transb"] = s["layout"].encode(), s["ta"].encode(), s["tb"].encode()
        p["m"], p["n"], p["k"] = s["m"], s["n"], s["k"]
        p["alpha"] = Q.scalar(s["al"])[0]
        p["beta"] = Q.scalar(s["be"])[0]
        p["A"], p["B"], p["C"] = ar.ptr(s["oA"]), ar.ptr(s["oB"]), ar.ptr(s["oC"])
        p["lda"], p["ldb"], p["ldc"] = s["lda"], s["ldb"], s["ldc"]
    return ar, specs, probs


def expected(O, s):
    al, be = Q.scalar(s["al"]), Q.scalar(s["be"])
    if s["op"] == 0:
        col, ta, tb = s["layout"] == "C", s["ta"] == "T", s["tb"] == "T"
        lda, ldb, ldc = s["lda"], s["ldb"], s["ldc"]
        if not col:
            sa = (1, lda) if ta else (lda, 1)
            sb = (1, ldb) if tb else (ldb, 1)
            sc = (ldc, 1)
        else:
            sa = (lda, 1) if ta else (1, lda)
            sb = (ldb, 1) if tb else (1, ldb)
            sc = (1, ldc)
        rows, cols = np.meshgrid(np.arange(s["m"]), np.arange(s["n"]), indexing="ij")
        rows, cols = rows.ravel(), cols.ravel()
        R, _, _ = O.exact_gemm(s["k"], s["A"], sa[0], sa[1], s["B"], sb[0], sb[1], rows, cols)
        idx = rows * sc[0] + cols * sc[1]
        out = s["C"].copy()
        out[idx] = epilogue(O, al, R, be, s["C"][idx])
        return out
    if s["op"] == 1:
        m, n = s["m"], s["n"]
        col = s["layout"] == "C"
        if s["ta"] == "T":
            m, n, col = n, m, not col
        si, sj = (1, s["lda"]) if col else (s["lda"], 1)
        R, _, _ = O.exact_gemv(m, n, s["A"], si, sj, s["B"], s["ldb"])
        out = s["C"].copy()
        out[::s["ldc"]][:m] = epilogue(O, al, R, be, s["C"][::s["ldc"]][:m])
        return out
    R, _, _ = O.exact_dot(s["A"], s["B"], s["n"], s["lda"], s["ldb"])
    return R


def check_all(O, ar, specs):
    got = ar.read()
    for s in specs:
        g = got[s["oC"]: s["oC"] + len(s["C"])]
        assert Q.same_bits(g, expected(O, s)).all(), (s["op"], s["m"], s["n"], s["k"], s["layout"], s["ta"])


@pytest.mark.parametrize("tile", [16, 32])
def test_batch_mixed_with_splits(qlib, O, torch_cuda, tile):
    torch = torch_cuda
    rng = G.rng_for(777)
    ar, specs, probs = make_batch(torch, rng, 40, 40, 40)
    api.batch_configure(1024, tile)  # tiny items: split-k, split rows and chunked dots
    try:
        plan = api.BatchPlan(probs)
        info = plan.info()
        assert info["split_groups"] > 0 and info["grain"] == 1024 and info["tile"] == tile
        plan.execute()
        torch.cuda.synchronize()
        check_all(O, ar, specs)
        plan.close()
    finally:
        api.batch_configure(1 << 16, 32)


def test_batch_reexecute_and_graph_replay(qlib, O, torch_cuda):
    torch = torch_cuda
    rng = G.rng_for(778)
    ar, specs, probs = make_batch(torch, rng, 20, 20, 20)
    for p in probs:  # beta = 0 everywhere so that repeated runs give the same outputs
        p["beta"] = Q.scalar(0.0)[0]
    for s in specs:
        s["be"] = 0.0
    api.batch_set_grain(2048)
    plan = api.BatchPlan(probs)
    plan.execute()
    torch.cuda.synchronize()
    first = ar.read().copy()
    check_all(O, ar, specs)
    plan.execute()
    torch.cuda.synchronize()
    assert Q.same_bits(ar.read(), first).all()
    # record the execution in a CUDA graph and replay it
    ar.dev.copy_(to_dev(torch, ar.all))
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        plan.execute(stream=s)
    g.replay()
    torch.cuda.synchronize()
    assert Q.same_bits(ar.read(), first).all()
    plan.close()


def test_batch_autotune(qlib, torch_cuda, tmp_path, monkeypatch):
    """Tile edge x granularity: the winner is in the candidate grid, set for
    new plans and appended to the cache file as "<device> <grain> <tile>"."""
    monkeypatch.setenv("QBLAS_AUTOTUNE_CACHE", str(tmp_path / "tune.txt"))
    g = api.batch_autotune()
    assert g in [1 << e for e in range(14, 21)]
    grain, tile = api.batch_setting()
    assert grain == g and tile in (16, 32)
    text = (tmp_path / "tune.txt").read_text().split()
    assert int(text[-2]) == g and int(text[-1]) == tile
    print({"grain": grain, "tile": tile})


def test_batch_ozaki_grouped_equals_single_calls(qlib, torch_cuda):
    """Under the Ozaki method, qgemm problems at or above the routing
    threshold run on the grouped residue path (stacked operands, one chain of
    launches over a tile list).  With the threshold at one product every
    qgemm problem of a mixed batch is routed (both layouts, all transposes,
    padded leading dimensions, beta != 0, a NaN and an infinity in two
    problems' operands); every output must equal, bit for bit, the same
    problems made one by one by quadblas_batch_run_serial, which gives the
    routed problems to the Ozaki single call (include/quadblas/algorithms/
    level3.hpp:215 semantics), also after a CUDA-graph replay."""
    torch = torch_cuda
    rng = G.rng_for(779)
    ar, specs, probs = make_batch(torch, rng, 40, 12, 12)
    gemms = [s for s in specs if s["op"] == 0]
    ar.dev[gemms[3]["oA"] + 2] = torch.tensor([0, 0x7FFF800000000000], dtype=torch.int64)   # NaN
    ar.dev[gemms[7]["oB"] + 1] = torch.tensor([0, -0x1000000000000], dtype=torch.int64)     # -inf (0xFFFF0000...)
    c0 = ar.dev.clone()
    api.set_method(2)
    api.batch_set_ozaki_min(1)
    try:
        plan = api.BatchPlan(probs)
        info = plan.info()
        assert info["ozaki_problems"] == len(gemms) and info["ozaki_tiles"] >= len(gemms)
        plan.execute()
        torch.cuda.synchronize()
        batched = ar.dev.clone()
        ar.dev.copy_(c0)
        torch.cuda.synchronize()
        api.batch_run_serial(probs)
        torch.cuda.synchronize()
        same = (batched == ar.dev).all(dim=1)
        assert bool(same.all()), int((~same).sum())
        # recorded in a CUDA graph and replayed
        ar.dev.copy_(c0)
        st = torch.cuda.Stream()
        st.wait_stream(torch.cuda.current_stream())
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=st):
            plan.execute(stream=st)
        g.replay()
        torch.cuda.synchronize()
        assert torch.equal(batched, ar.dev)
        plan.close()
    finally:
        api.set_method(0)
        api.batch_set_ozaki_min(0)


def test_batch_ozaki_grouped_multi_tile_problems(qlib, torch_cuda):
    """Routed qgemm problems that span several 128 x 256 tiles in both
    directions (so tiles start at local rows and columns other than 0),
    longer k (several exact 256-chunks, k_pad set by the largest k), a
    column-major C with a padded leading dimension, and a problem below the
    threshold that stays on the persistent kernel: bit-identical to the
    single calls made by quadblas_batch_run_serial."""
    torch = torch_cuda
    rng = G.rng_for(780)
    shapes = [(300, 600, 700, "R", "N", "N"), (130, 257, 1000, "C", "T", "N"), (1, 1000, 9, "R", "N", "T"),
              (257, 3, 2049, "C", "N", "T"), (20, 20, 20, "R", "N", "N")]
    ar = Arena(torch)
    specs = []
    for m, n, k, layout, ta, tb in shapes:
        col = layout == "C"
        a_r, a_c = (k, m) if ta == "T" else (m, k)
        b_r, b_c = (n, k) if tb == "T" else (k, n)
        lda, ldb = (a_r if col else a_c) + 1, (b_r if col else b_c) + 2
        ldc = (m if col else n) + 3
        A = G.spread_uniform(rng, (a_c if col else a_r) * lda)
        B = G.spread_uniform(rng, (b_c if col else b_r) * ldb)
        C = G.uniform_full(rng, (n if col else m) * ldc)
        specs.append(dict(m=m, n=n, k=k, layout=layout, ta=ta, tb=tb, lda=lda, ldb=ldb, ldc=ldc,
                          oA=ar.add(A), oB=ar.add(B), oC=ar.add(C)))
    ar.upload()
    probs = np.zeros(len(specs), dtype=api.PROBLEM_DTYPE)
    for p, s in zip(probs, specs):
        p["op"] = api.OP_GEMM
        p["layout"], p["transa"], p["transb"] = s["layout"].encode(), s["ta"].encode(), s["tb"].encode()
        p["m"], p["n"], p["k"] = s["m"], s["n"], s["k"]
        p["alpha"], p["beta"] = Q.scalar(1.5)[0], Q.scalar(-0.25)[0]
        p["A"], p["B"], p["C"] = ar.ptr(s["oA"]), ar.ptr(s["oB"]), ar.ptr(s["oC"])
        p["lda"], p["ldb"], p["ldc"] = s["lda"], s["ldb"], s["ldc"]
    c0 = ar.dev.clone()
    api.set_method(2)
    api.batch_set_ozaki_min(20 * 20 * 20 + 1)
    try:
        plan = api.BatchPlan(probs)
        info = plan.info()
        assert info["ozaki_problems"] == len(shapes) - 1
        assert info["ozaki_tiles"] == 3 * 3 + 2 * 2 + 1 * 4 + 3 * 1
        plan.execute()
        torch.cuda.synchronize()
        batched = ar.dev.clone()
        ar.dev.copy_(c0)
        torch.cuda.synchronize()
        api.batch_run_serial(probs)
        torch.cuda.synchronize()
        same = (batched == ar.dev).all(dim=1)
        assert bool(same.all()), int((~same).sum())
        plan.close()
    finally:
        api.set_method(0)
        api.batch_set_ozaki_min(0)


def test_batched_dev_one_shot(qlib, O, torch_cuda):
    """quadblas_qgemm_batched_dev (plan, execute, wait, free in one call) on a
    mixed batch: every output equal to the exact oracle's single-call result;
    under the Ozaki method with every qgemm problem routed, equal to the
    one-by-one calls."""
    torch = torch_cuda
    rng = G.rng_for(781)
    ar, specs, probs = make_batch(torch, rng, 10, 10, 10)
    c0 = ar.dev.clone()
    api.batched_dev(probs)
    torch.cuda.synchronize()
    check_all(O, ar, specs)
    api.set_method(2)
    api.batch_set_ozaki_min(1)
    try:
        ar.dev.copy_(c0)
        api.batched_dev(probs)
        torch.cuda.synchronize()
        batched = ar.dev.clone()
        ar.dev.copy_(c0)
        api.batch_run_serial(probs)
        torch.cuda.synchronize()
        assert torch.equal(batched, ar.dev)
    finally:
        api.set_method(0)
        api.batch_set_ozaki_min(0)
