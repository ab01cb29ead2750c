"""Benchmark of the binary128 hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload qgemm4096|qgemm512|qgemv8192|qdot26]

Default workload: qgemm m = n = k = 4096, row-major 'N','N', alpha = 1,
beta = 0, entries u * 2^e (u uniform in [-1, 1) with full 113-bit
significand, e uniform in [-20, 20]); the metric is binary128 GFLOP/s
(2mnk per second).  One step is one qgemm with inputs resident in HBM.
The qgemv 8192^2 and qdot 2^26 HBM workloads are measured beside it
("secondary").  Each rank runs its own problem (weak scaling; the paths
need no collective), rank 0 prints one JSON line.

--impl reference times the reference's CPU algorithm (the oracle's
restatement of QuadBLAS's blocked gemm, OpenMP over all host cores) on a
bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from qblas_gb300 import gen as G  # noqa: E402
from qblas_gb300 import quad as Q  # noqa: E402

L2_BYTES = 129 * 2**20
FALLBACK = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return d, "measured"
    except (OSError, ValueError):
        return dict(FALLBACK), "fallback"


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.dev)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        if not getattr(self, "lines", None):
            return None
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [s.strip() for s in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        load = [s for s in sm if s > 0.5 * max(sm)]
        return {"sm_mhz": statistics.median(load or sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# workloads (ours)
# ---------------------------------------------------------------------------
def dev_tensor(torch, a: np.ndarray):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int64)).cuda()


def time_steps(torch, fn, steps, warmup, dist=None):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(steps):
        fn()
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    if dist is not None:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        dist.barrier()
    return ms


class Qgemm:
    def __init__(self, torch, m, n, k, seed, spread=True):
        from qblas_gb300 import api
        self.torch, self.api = torch, api
        self.m, self.n, self.k = m, n, k
        rng = G.rng_for(seed)
        if spread:
            self.A, self.B = G.spread_uniform(rng, m * k), G.spread_uniform(rng, k * n)
        else:
            self.A, self.B = G.uniform_full(rng, m * k), G.uniform_full(rng, k * n)
        self.C = Q.from_double(np.zeros(m * n))
        self.dA, self.dB, self.dC = dev_tensor(torch, self.A), dev_tensor(torch, self.B), dev_tensor(torch, self.C)
        self.alpha, self.beta = Q.scalar(1.0), Q.scalar(0.0)

    def flops(self):
        return 2.0 * self.m * self.n * self.k

    def step(self):
        self.api.gemm_dev("R", "N", "N", self.m, self.n, self.k, self.alpha, self.dA, self.k, self.dB, self.n,
                          self.beta, self.dC, self.n)

    def launches_per_step(self):
        return 1

    def e2e(self, steps):
        torch, api = self.torch, self.api
        pin = lambda a: torch.from_numpy(a.view(np.int64)).pin_memory().numpy().view(np.uint64)  # noqa: E731
        hA, hB, hC = pin(self.A), pin(self.B), pin(self.C)
        api.gemm("R", "N", "N", self.m, self.n, self.k, self.alpha, hA, self.k, hB, self.n, self.beta, hC, self.n)
        t0 = time.perf_counter()
        for _ in range(steps):
            api.gemm("R", "N", "N", self.m, self.n, self.k, self.alpha, hA, self.k, hB, self.n, self.beta, hC,
                     self.n)
        dt = time.perf_counter() - t0
        h2d = (self.A.size + self.B.size + self.C.size) * 8
        d2h = self.C.size * 8
        return dt / steps, h2d, d2h


class Qgemv:
    def __init__(self, torch, m, n, seed):
        from qblas_gb300 import api
        self.torch, self.api, self.m, self.n = torch, api, m, n
        rng = G.rng_for(seed)
        self.dA = dev_tensor(torch, G.wide_exponent(rng, m * n))
        self.dx = dev_tensor(torch, G.wide_exponent(rng, n))
        self.dy = dev_tensor(torch, G.wide_exponent(rng, m))
        self.alpha, self.beta = Q.scalar(1.0), Q.scalar(0.0)

    def bytes(self):
        return 16.0 * (self.m * self.n + self.n + self.m)

    def step(self):
        self.api.gemv_dev("R", "N", self.m, self.n, self.alpha, self.dA, self.n, self.dx, 1, self.beta, self.dy, 1)


class Qdot:
    def __init__(self, torch, n, seed):
        from qblas_gb300 import api
        self.torch, self.api, self.n = torch, api, n
        x, y = G.cancelling_dot(G.rng_for(seed), n)
        self.dx, self.dy = dev_tensor(torch, x), dev_tensor(torch, y)
        self.dr = torch.zeros((1, 2), dtype=torch.int64, device="cuda")

    def bytes(self):
        return 32.0 * self.n

    def step(self):
        self.api.dot_dev(self.n, self.dx, 1, self.dy, 1, self.dr)


def hbm_roofline(pk, src, nbytes, ms_per_launch):
    gbs = nbytes / (ms_per_launch * 1e-3) / 1e9
    peak = float(pk.get("hbm_gbs", FALLBACK["hbm_gbs"]))
    return {"bound": "hbm", "achieved": round(gbs, 1), "peak": peak, "unit": "GB/s", "frac": round(gbs / peak, 4),
            "traffic": None, "peak_source": src}


# ---------------------------------------------------------------------------
# CPU baseline: the oracle's restatement of the reference (OpenMP)
# ---------------------------------------------------------------------------
def cpu_gemm_sample(target_s=12.0):
    """Reference-order blocked qgemm (k = 4096, k-panels of 126) on an m x n
    slice sized for about target_s seconds on all host cores."""
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    k = 4096
    rng = G.rng_for(77)

    def run(mm, nn):
        A, B = G.spread_uniform(rng, mm * k), G.spread_uniform(rng, k * nn)
        C = Q.from_double(np.zeros(mm * nn))
        t0 = time.perf_counter()
        O.ref_gemm(0, mm, nn, k, Q.scalar(1.0), A, k, B, nn, Q.scalar(0.0), C, nn, lib_order=1, nthreads=cores)
        return time.perf_counter() - t0

    mm = nn = 16
    t = run(mm, nn)
    rate = (mm * nn) / max(t, 1e-6)
    side = int(np.sqrt(rate * target_s))
    side = max(16, min(side, 1024))
    t = run(side, side)
    gflops = 2.0 * side * side * k / t / 1e9
    return {"value": gflops, "unit": "GFLOP/s", "cores": cores, "kind": "port",
            "sample": f"qgemm {side}x{side}x{k} (reference blocked order, kc=126) in {t:.1f} s, "
                      f"OpenMP {cores} threads"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    base = None
    times = []
    for _ in range(max(args.warmup, 0) and 1):
        cpu_gemm_sample(target_s=3.0)
    for _ in range(args.steps):
        base = cpu_gemm_sample(target_s=8.0)
        times.append(base["value"])
    v = statistics.median(times)
    line = {"metric": "qgemm binary128 GFLOP/s (4096^3 workload)", "value": round(v, 6), "unit": "GFLOP/s",
            "impl": "reference", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "binary128 (host long double / __float128 FMA)", "data": "synthetic",
            "config": {"workload": "qgemm m=n=k=4096 row-major NN alpha=1 beta=0 (sampled m x n slice, full k)"},
            "cpu_baseline": {"value": round(v, 6), "unit": "GFLOP/s", "cores": base["cores"], "kind": "port",
                             "sample": base["sample"]},
            "e2e": {"value": round(v, 6), "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="qgemm4096", choices=["qgemm4096", "qgemm512", "qgemv8192", "qdot26"])
    ap.add_argument("--method", default="softfloat", choices=["softfloat", "ozaki"])
    ap.add_argument("--slices", type=int, default=0)
    ap.add_argument("--no-secondary", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as td
        td.init_process_group("nccl")
        dist = td
    from qblas_gb300 import _lib, api
    _lib.load()
    pk, pk_src = peaks()
    api.set_method(2 if args.method == "ozaki" else 1)
    api.set_ozaki_slices(args.slices)

    wl = args.workload
    if wl.startswith("qgemm"):
        size = 4096 if wl == "qgemm4096" else 512
        W = Qgemm(torch, size, size, size, seed=0xC0FFEE + 2 + rank, spread=(size == 4096))
        with ClockSampler(local) as clk:
            ms = time_steps(torch, W.step, args.steps, args.warmup, dist)
        ms_step = ms / args.steps
        value = world * W.flops() / (ms_step * 1e-3) / 1e9
        metric, unit = f"qgemm binary128 GFLOP/s ({size}^3)", "GFLOP/s"
        launches = W.launches_per_step() * args.steps
        # soft-float qgemm: one kernel per step, so the step time is the kernel time
        roof = {"bound": "int", "achieved": round(W.flops() / (ms_step * 1e-3) / 1e9, 3),
                "peak": None, "unit": "quad GFLOP/s", "frac": None, "traffic": None,
                "note": "soft-float kernel is integer-pipe bound; no tensor/HBM roofline applies"}
        e2e_s, h2d, d2h = W.e2e(max(1, min(args.steps, 3)))
        e2e = {"value": round(W.flops() / e2e_s / 1e9, 3), "unit": unit, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h)}
        cfg = {"workload": f"qgemm m=n=k={size} row-major NN alpha=1 beta=0, entries u*2^e "
                           f"(u uniform [-1,1) full 113-bit significand, e uniform [-20,20])" if size == 4096 else
                           f"qgemm m=n=k={size} row-major NN alpha=1 beta=0, full-mantissa uniform [-1,1)",
               "method": args.method, "l2": "inputs larger than L2 (no flush)" if size == 4096 else
               "inputs fit in L2; one launch per step", "parallelism": f"replicas x{world}"}
        dtype = "u32 (soft-float integer limbs)"
    elif wl == "qgemv8192":
        W = Qgemv(torch, 8192, 8192, seed=11 + rank)
        with ClockSampler(local) as clk:
            ms = time_steps(torch, W.step, args.steps, args.warmup, dist)
        ms_step = ms / args.steps
        value = world * W.bytes() / (ms_step * 1e-3) / 1e9
        metric, unit = "qgemv binary128 GB/s (8192^2 row-major)", "GB/s"
        launches = args.steps
        roof = hbm_roofline(pk, pk_src, W.bytes(), ms_step)
        e2e, cfg, dtype = None, {"workload": "qgemv 8192x8192 row-major alpha=1 beta=0 wide-exponent"}, "u32"
    else:
        W = Qdot(torch, 1 << 26, seed=13 + rank)
        with ClockSampler(local) as clk:
            ms = time_steps(torch, W.step, args.steps, args.warmup, dist)
        ms_step = ms / args.steps
        value = world * W.bytes() / (ms_step * 1e-3) / 1e9
        metric, unit = "qdot binary128 GB/s (n=2^26)", "GB/s"
        launches = 2 * args.steps
        roof = hbm_roofline(pk, pk_src, W.bytes(), ms_step)
        e2e, cfg, dtype = None, {"workload": "qdot n=2^26 wide-exponent with cancelling pairs"}, "u32"

    secondary = {}
    if not args.no_secondary and wl == "qgemm4096":
        del W
        torch.cuda.empty_cache()
        for name, mk, unitb in [("qgemv8192", lambda: Qgemv(torch, 8192, 8192, 11 + rank), "GB/s"),
                                ("qdot26", lambda: Qdot(torch, 1 << 26, 13 + rank), "GB/s")]:
            S = mk()
            ms2 = time_steps(torch, S.step, args.steps, 3, dist) / args.steps
            secondary[name] = {"value": round(S.bytes() / (ms2 * 1e-3) / 1e9, 1), "unit": unitb,
                               "ms_per_step": round(ms2, 4), "roofline": hbm_roofline(pk, pk_src, S.bytes(), ms2)}
            del S
            torch.cuda.empty_cache()
        S = Qgemm(torch, 512, 512, 512, seed=0xC0FFEE, spread=False)
        ms2 = time_steps(torch, S.step, 20, 3, dist) / 20
        secondary["qgemm512_softfloat"] = {"value": round(S.flops() / (ms2 * 1e-3) / 1e9, 3), "unit": "GFLOP/s",
                                           "ms_per_step": round(ms2, 4)}

    cpu = None
    if rank == 0 and not args.no_cpu and wl.startswith("qgemm"):
        cpu = cpu_gemm_sample()
        cpu["value"] = round(cpu["value"], 6)

    if rank == 0:
        line = {"metric": metric, "value": round(value, 3), "unit": unit, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(ms_step, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic (seeded)",
                "config": cfg, "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
                "clocks": clk.summary(), "gpu_launches": launches}
        if secondary:
            line["secondary"] = secondary
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
