"""The multi-rank path of bench.py, run on the CPU as two gloo ranks
(world_size 2, rendezvous on 127.0.0.1): every rank gets the slowest rank's
time, the whole-job rate counts the units of all ranks over that time, and
the reference arm prints only on rank 0."""
import os
import socket
import subprocess
import sys

import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as td
    td.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    import bench
    slowest = bench.max_over_ranks(td, 10.0 + 3.0 * rank)
    td.barrier()
    q.put((rank, slowest, bench.whole_job_rate(100.0, world, slowest)))
    td.destroy_process_group()


def test_max_over_ranks_and_whole_job_rate_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=180) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, _, _ in res] == [0, 1]
    assert all(t == 13.0 for _, t, _ in res)
    assert all(abs(v - 2 * 100.0 / 13.0) < 1e-12 for _, _, v in res)


def test_single_rank_has_no_collective():
    import bench
    assert bench.max_over_ranks(None, 7.5) == 7.5
    assert bench.whole_job_rate(10.0, 1, 2.0) == 5.0


def test_reference_arm_prints_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                         env=env, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.strip() == ""
