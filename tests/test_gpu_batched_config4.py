"""GPU parity of the batched launch on the full batched workload.

10,000 qgemm problems (m, n, k log-uniform in [8, 256]), 10,000 qgemv
problems (m, n log-uniform in [16, 2048]) and 10,000 qdot problems (n
log-uniform in [64, 65536]), row-major 'N', alpha = 1, beta = 0, with
full-mantissa uniform values: the shapes and item sizes (split-k tiles,
column-split rows, chunked dots) that the benchmark runs, not a reduced
case.  The batch goes through the autotuned plan, recorded in a CUDA graph
and replayed.  At the autotuned granularity no item of this workload is
split, so the batch is also planned with the other qgemm tile edge (16 or
32) and at granularity 2^14, where qgemm tiles split along k, long qgemv rows
along the columns and long dots into chunks; those executions must give the
same bits.

Every output must be bit-identical to the same problem run by its own
device-pointer call (quadblas_batch_run_serial): both claim the correctly
rounded sum through the single-call epilogue, so no tolerance applies.  A
seeded sample of 100 problems of each kind is checked against the exact
oracle as well.  Per-problem semantics: QuadBLAS::gemm
(include/quadblas/algorithms/level3.hpp:215), QuadBLAS::gemv
(level2.hpp:85), QuadBLAS::dot (level1.hpp:80).
"""
import numpy as np
import pytest

from gpu_helpers import epilogue
from qblas_gb300 import api
from qblas_gb300 import gen as G
from qblas_gb300 import quad as Q

pytestmark = pytest.mark.gpu


def _host(t, off, cnt):
    return np.ascontiguousarray(t[int(off): int(off) + int(cnt)].cpu().numpy()).view(np.uint64)


def test_config4_batched_equals_one_by_one_and_oracle(qlib, O, torch_cuda, tmp_path, monkeypatch):
    torch = torch_cuda
    monkeypatch.setenv("QBLAS_AUTOTUNE_CACHE", str(tmp_path / "tune.txt"))
    probs, inp, out, lay = G.config4_batch(torch, 4000)
    c0 = out.clone()
    api.set_method(1)
    try:
        grain = api.batch_autotune()
        plan = api.BatchPlan(probs)
        info = plan.info()
        assert info["grain"] == grain
        st = torch.cuda.Stream()
        st.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(st):
            plan.execute(stream=st)  # warm-up outside the graph
            torch.cuda.synchronize()
            out.copy_(c0)
            torch.cuda.synchronize()
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graph, stream=st):
                plan.execute(stream=st)
        torch.cuda.synchronize()
        out.copy_(c0)
        graph.replay()
        torch.cuda.synchronize()
        batched = out.clone()
        # the same problems, one call each, from the original C values
        out.copy_(c0)
        torch.cuda.synchronize()
        api.batch_run_serial(probs)
        torch.cuda.synchronize()
        if not torch.equal(batched, out):
            diff = (batched != out).any(dim=1).nonzero().flatten().cpu().numpy()
            bad = sorted({i for i, L in enumerate(lay) if np.any((diff >= L[6]) & (diff < L[6] + L[7]))})
            pytest.fail(f"{diff.size} outputs differ, in {len(bad)} problems, first {[lay[i][:4] for i in bad[:5]]}")
        plan.close()
        del graph
        # the other gemm tile edge at the same granularity
        _, tile = api.batch_setting()
        api.batch_configure(grain, 48 - tile)
        plan = api.BatchPlan(probs)
        assert plan.info()["tile"] == 48 - tile
        out.copy_(c0)
        plan.execute()
        torch.cuda.synchronize()
        assert torch.equal(batched, out), f"tile {48 - tile} execution differs"
        plan.close()
        # small items: split-k tiles, column-split rows, chunked dots, merged in order
        api.batch_set_grain(1 << 14)
        plan = api.BatchPlan(probs)
        assert plan.info()["split_groups"] > 0
        out.copy_(c0)
        plan.execute()
        torch.cuda.synchronize()
        assert torch.equal(batched, out), "split-item execution differs"
        plan.close()
    finally:
        api.set_method(0)
        api.batch_configure(1 << 16, 32)

    # a seeded sample of each kind against the exact oracle
    rng = np.random.default_rng(44)
    one, zero = Q.scalar(1.0), Q.scalar(0.0)
    for op, lo in ((0, 0), (1, 10000), (2, 20000)):
        for i in rng.choice(10000, 100, replace=False) + lo:
            _, m, n, k, a, b, c, lc = lay[i]
            got = _host(batched, c, lc)
            cold = _host(c0, c, lc)
            if op == 0:
                A, B = _host(inp, a, m * k), _host(inp, b, k * n)
                rows, cols = np.meshgrid(np.arange(m), np.arange(n), indexing="ij")
                R, _, _ = O.exact_gemm(k, A, k, 1, B, n, 1, rows.ravel(), cols.ravel())
            elif op == 1:
                A, x = _host(inp, a, m * n), _host(inp, b, n)
                R, _, _ = O.exact_gemv(m, n, A, n, 1, x, 1)
            else:
                x, y = _host(inp, a, n), _host(inp, b, n)
                R, _, _ = O.exact_dot(x, y)
                assert Q.same_bits(got, R).all(), (op, n)
                continue
            assert Q.same_bits(got, epilogue(O, one, R, zero, cold)).all(), (op, m, n, k)


def test_config4_ozaki_routing_equals_one_by_one(qlib, torch_cuda, tmp_path, monkeypatch):
    """The same workload under the Ozaki method: the qgemm problems with
    m n k >= 2^20 (the default threshold) run on the grouped residue path,
    the rest of the batch on the persistent kernel.  Every output must be
    bit-identical to quadblas_batch_run_serial, which makes the Ozaki single
    call for the routed problems and the soft-float call for the others."""
    torch = torch_cuda
    monkeypatch.setenv("QBLAS_AUTOTUNE_CACHE", str(tmp_path / "tune.txt"))
    probs, inp, out, lay = G.config4_batch(torch, 4001)
    c0 = out.clone()
    api.set_method(2)
    api.batch_set_ozaki_min(0)
    try:
        plan = api.BatchPlan(probs)
        info = plan.info()
        routed = sum(1 for L in lay if L[0] == 0 and L[1] * L[2] * L[3] >= 1 << 20)
        assert info["ozaki_problems"] == routed > 0
        plan.execute()
        torch.cuda.synchronize()
        batched = out.clone()
        out.copy_(c0)
        torch.cuda.synchronize()
        api.batch_run_serial(probs)
        torch.cuda.synchronize()
        same = (batched == out).all(dim=1)
        if not bool(same.all()):
            diff = (~same).nonzero().flatten().cpu().numpy()
            bad = sorted({i for i, L in enumerate(lay) if np.any((diff >= L[6]) & (diff < L[6] + L[7]))})
            pytest.fail(f"{diff.size} outputs differ, in {len(bad)} problems, first {[lay[i][:4] for i in bad[:5]]}")
        plan.close()
    finally:
        api.set_method(0)
