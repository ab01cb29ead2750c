"""Benchmark of the binary128 hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload qgemm4096|qgemm2048|qgemm512|qgemv8192|qdot26]
                    [--method ozaki|softfloat] [--slices S] [--bits B]
                    [--scheme auto|digits|residues]

Default: qgemm m = n = k = 4096, row-major 'N','N', alpha = 1, beta = 0,
entries u * 2^e (u uniform in [-1, 1) with a full 113-bit significand, e a
uniform integer in [-20, 20]), Ozaki method with each operand truncated to
T = 9 * 15 - 1 = 134 bits after its row (column) scaling, multiplied by the
automatic scheme: residues modulo 32 coprime moduli (Ozaki scheme II, one
fp16 tensor-core GEMM per modulus, exact CRT reconstruction; <= 1 ulp on
this workload); metric binary128 GFLOP/s (2mnk per second).  One step is
one qgemm with the inputs resident in HBM (A and B are 256 MB each, larger
than L2, so no flush is needed).  Beside it ("secondary"): the soft-float
qgemm of the same problem (the speed-up of the Ozaki path over it), a
sweep over T and both schemes with the ulp distance of each result from
the correctly rounded soft-float result, the library's default setting,
qgemv 8192^2 and qdot 2^26 (HBM rooflines), the 30,000-problem batch
(soft-float, and under the Ozaki method with large qgemm problems on the
grouped residue path) and the 512^3 soft-float qgemm.

Each rank runs its own problem (weak scaling; the path needs no
collective); rank 0 prints one JSON line.

--impl reference times the reference's CPU algorithm (the oracle's
restatement of QuadBLAS's blocked gemm, OpenMP over all host cores) on a
bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes
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

FALLBACK = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}
# (scheme, digit bits, digits): the truncation is T = bits * digits - 1 bits
# per operand; "digits" multiplies digit pairs, "residues" moduli (CRT)
SWEEP = (("residues", 9, 11), ("residues", 9, 12), ("residues", 9, 13), ("residues", 9, 14),
         ("residues", 9, 15), ("residues", 9, 16), ("residues", 9, 18), ("residues", 8, 20),
         ("digits", 8, 12), ("digits", 8, 16), ("digits", 8, 17), ("digits", 9, 14), ("digits", 9, 15))
SCHEMES = {"auto": 0, "digits": 1, "residues": 2}
HEADLINE_DIGITS, HEADLINE_BITS = 15, 9  # <= 1 ulp on this workload (tests/test_gpu_ozaki.py)


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return json.load(f), "measured"
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
        self.lines = []

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
        sm, mx, power, reasons = [], 0.0, [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [s.strip() for s in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        load = [s for s in sm if s > 0.5 * max(sm)]
        return {"sm_mhz": statistics.median(load or sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "power_w_max": max(power) if power else None, "samples": len(sm)}


# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------
def dev_tensor(torch, a: np.ndarray):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int64)).cuda()


def to_host(t) -> np.ndarray:
    return np.ascontiguousarray(t.cpu().numpy()).view(np.uint64)


def ozaki_launches(k, s, b, crt):
    """Kernels per device-pointer Ozaki qgemm call on one stream, square and
    row-major: one kernel setting the scales' starting values and error words,
    op(B)'s scale and split, op(A)'s split (residues: op(A)'s scales come from
    a side warp of op(B)'s split; digit pairs: a scale launch of their own),
    one tensor-core launch per k pass (residues over several passes: one more
    summing them), fold, special values.  Digit pairs: a k pass holds as many
    fp32-exact k-chunks as an int32 diagonal sum of s pairs of chunk sums
    (each < 2^24) allows.  Residues: a k pass is 8192 (the residue product
    sums stay below 2^29)."""
    if crt:
        npass = -(-k // 8192)
        return 4 + npass + (1 if npass > 1 else 0) + 2
    chunk_kb = (1 << (24 - 2 * (b - 1))) // 64
    kbp = max(1, (2 ** 31 - 1) // (s << 24)) * chunk_kb
    npass = -(-(-(-k // 64)) // kbp)
    return 5 + npass + 2


def max_over_ranks(dist, x: float) -> float:
    """The largest x over all ranks (x itself without a process group).  The
    reduction runs on the GPU under NCCL and on the CPU under gloo."""
    if dist is None:
        return float(x)
    import torch
    dev = "cpu" if dist.get_backend() == "gloo" else "cuda"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world: int, seconds: float) -> float:
    """Units per second of the whole job: every rank processes units_per_rank
    (weak scaling) and the job takes the slowest rank's time."""
    return world * units_per_rank / seconds


def time_steps(torch, fn, steps, warmup, dist=None):
    """CUDA-event time (ms) of `steps` calls on the current stream, max over ranks."""
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
    ms = max_over_ranks(dist, e0.elapsed_time(e1))
    if dist is not None:
        dist.barrier()
    return ms


def ulp_distance(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """|a - b| in binary128 ulps (distance in the ordered bit patterns)."""
    def key(q):
        out = []
        for lo, hi in q:
            v = (int(hi) << 64) | int(lo)
            mag = v & ((1 << 127) - 1)
            out.append(-mag if v >> 127 else mag)
        return out
    ka, kb = key(a), key(b)
    return np.array([abs(x - y) for x, y in zip(ka, kb)], dtype=np.float64)


def relative_error(a: np.ndarray, ref: np.ndarray) -> np.ndarray:
    """|a - ref| / |ref| for binary128 values, from the ulp distance and the
    significand of ref (ulp(ref) / |ref| = 2^-112 / 1.f)."""
    d = ulp_distance(a, ref)
    f = 1.0 + (ref[:, 1] & np.uint64((1 << 48) - 1)).astype(np.float64) / float(1 << 48)
    return d * 2.0 ** -112 / f


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

    def e2e(self, steps, pinned=True):
        """Public host-pointer API (quadblas_qgemm_q): H2D of A, B, C and D2H of C
        inside the timed region, from pinned host memory or (pinned=False) from
        ordinary pageable memory, as a reference caller's Matrix<L> allocates
        it (posix_memalign, include/quadblas/memory/allocation.hpp:25)."""
        torch, api = self.torch, self.api
        if pinned:
            pin = lambda a: torch.from_numpy(a.view(np.int64)).pin_memory().numpy().view(np.uint64)  # noqa: E731
        else:
            pin = lambda a: np.array(a, copy=True)  # noqa: E731
        hA, hB, hC = pin(self.A), pin(self.B), pin(self.C)
        api.gemm("R", "N", "N", self.m, self.n, self.k, self.alpha, hA, self.k, hB, self.n, self.beta, hC, self.n)
        t0 = time.perf_counter()
        for _ in range(steps):
            api.gemm("R", "N", "N", self.m, self.n, self.k, self.alpha, hA, self.k, hB, self.n, self.beta, hC,
                     self.n)
        dt = time.perf_counter() - t0
        return dt / steps, (self.A.size + self.B.size + self.C.size) * 8, self.C.size * 8


class Qgemv:
    def __init__(self, torch, m, n, seed):
        from qblas_gb300 import api
        self.api, self.m, self.n = api, m, n
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
        self.api, self.n = api, n
        x, y = G.cancelling_dot(G.rng_for(seed), n)
        self.dx, self.dy = dev_tensor(torch, x), dev_tensor(torch, y)
        self.dr = torch.zeros((1, 2), dtype=torch.int64, device="cuda")

    def bytes(self):
        return 32.0 * self.n

    def step(self):
        self.api.dot_dev(self.n, self.dx, 1, self.dy, 1, self.dr)


# DRAM bytes (read + write) per launch of the dominant kernel, from one ncu
# capture of the same workload (profiles/ holds the summaries and commands).
NCU_TRAFFIC = {
    "qgemm4096": (2 * (9.84e9 + 1.01e9), "profiles/ozaki_mma_kernel_4096_traffic.md"),  # 15 x 9 bit digit pairs, 2 passes
    "qgemm4096_crt": (2.978e9 + 1.054e9, "profiles/ozaki_crt_qgemm4096_launches.md"),  # T = 134, 32 moduli
    "qdot26": (2.147608e9 + 4.091e6, "profiles/qdot_partial_kernel_n2p26.md"),
    "qgemv8192": (1.074079e9 + 1.8140e7, "profiles/qgemv_lane_kernel_8192.md"),
    "qgemv8192_ozaki": (1.086039e9 + 3.946e6, "profiles/og_gemv_kernel_8192.md"),
}


def traffic(workload):
    """(DRAM bytes per launch of the dominant kernel, the profile it comes from)."""
    t = NCU_TRAFFIC.get(workload)
    return (t[0], t[1]) if t else (None, None)


def hbm_roofline(pk, src, nbytes, ms_per_launch, workload=None):
    gbs = nbytes / (ms_per_launch * 1e-3) / 1e9
    peak = float(pk.get("hbm_gbs", FALLBACK["hbm_gbs"]))
    tb, ts = traffic(workload)
    return {"bound": "hbm", "achieved": round(gbs, 1), "peak": peak, "unit": "GB/s", "frac": round(gbs / peak, 4),
            "traffic": tb, "traffic_source": ts, "algorithmic_bytes": nbytes, "peak_source": src}


def batched_config4(torch, api, rank, reps=3):
    """10,000 qgemm (m, n, k log-uniform in [8, 256]), 10,000 qgemv (m, n in
    [16, 2048]) and 10,000 qdot (n in [64, 65536]) with full-mantissa uniform
    values, row-major 'N', alpha = 1, beta = 0: one persistent launch (CUDA
    graph replay) against the same problems launched one device-pointer call
    at a time from a C loop (quadblas_batch_run_serial).  Outside the timed
    regions the two sets of outputs are compared bit for bit (both are the
    correctly rounded sums)."""
    probs, inp, out, lay = G.config4_batch(torch, 4000 + rank)
    flops = 0.0
    for op, m, n, k, *_ in lay:
        flops += 2.0 * (m * n * k if op == 0 else (m * n if op == 1 else n))
    c0 = out.clone()
    # gemm tile edge and work-item granularity come from the autotuner
    t0 = time.perf_counter()
    api.batch_autotune()
    tune_s = time.perf_counter() - t0
    grain, tile = api.batch_setting()
    t0 = time.perf_counter()
    plan = api.BatchPlan(probs)
    plan_s = time.perf_counter() - t0
    info = plan.info()
    st = torch.cuda.Stream()
    st.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(st):
        plan.execute(stream=st)
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=st):
            plan.execute(stream=st)
    torch.cuda.synchronize()
    graph.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        graph.replay()
    e1.record()
    torch.cuda.synchronize()
    ms_batched = e0.elapsed_time(e1) / reps
    out.copy_(c0)
    graph.replay()
    torch.cuda.synchronize()
    batched = out.clone()
    # the same problems, one library call each from a C loop, on the current stream
    api.batch_run_serial(probs)  # warm-up (the scratch pool grows to need)
    torch.cuda.synchronize()
    out.copy_(c0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e0.record()
    api.batch_run_serial(probs)
    e1.record()
    torch.cuda.synchronize()
    wall_single = time.perf_counter() - t0
    ms_single = max(e0.elapsed_time(e1), wall_single * 1e3)
    same = bool(torch.equal(batched, out))
    plan.close()
    del graph, inp, out, c0, batched
    torch.cuda.empty_cache()
    return {"problems": len(probs), "gflops": round(flops / (ms_batched * 1e-3) / 1e9, 2),
            "ms_batched_graph_replay": round(ms_batched, 3), "ms_one_call_per_problem": round(ms_single, 3),
            "one_by_one": "quadblas_batch_run_serial (C loop of device-pointer calls)",
            "speedup_vs_one_by_one": round(ms_single / ms_batched, 2), "plan_ms": round(plan_s * 1e3, 1),
            "work_items": info["items"], "grain": info["grain"], "tile": info["tile"],
            "autotuned": {"grain": grain, "tile": tile, "candidates": "tile {16, 32} x grain 2^14..2^20"},
            "autotune_ms": round(tune_s * 1e3, 1), "launches_per_batch": 1,
            "parity": "bit-identical to one-by-one" if same else "MISMATCH against one-by-one",
            "method_mix": {"softfloat_wide_accumulator": len(probs) - info["ozaki_problems"],
                           "ozaki_grouped_residues": info["ozaki_problems"], "ozaki_tiles": info["ozaki_tiles"]},
            "quad_flops": flops}


def oracle_accuracy(W, C, rank, samples=512):
    """Max ulp and max relative error of the qgemm result C against the exact
    oracle (correctly rounded exact sums) on a seeded sample of entries;
    runs after the timed region (the oracle checks, it is not measured)."""
    from oracle import oracle as O
    O.build()
    rng = np.random.default_rng(900 + rank)
    rows = rng.integers(0, W.m, samples)
    cols = rng.integers(0, W.n, samples)
    R, _, _ = O.exact_gemm(W.k, W.A, W.k, 1, W.B, W.n, 1, rows, cols)
    got = C[rows * W.n + cols]
    d = ulp_distance(got, R)
    return {"max": float(d.max()), "max_rel": float(relative_error(got, R).max()),
            "exact_frac": float((d == 0).mean()), "samples": int(samples),
            "reference": "exact oracle (Kulisch accumulator, correctly rounded)"}


def profile_read(lib):
    out = (ctypes.c_double * 4)()
    calls = ctypes.c_int(0)
    lib.quadblas_profile_read(out, ctypes.byref(calls))
    return list(out), calls.value


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

    t = run(16, 16)
    rate = 256 / max(t, 1e-6)
    side = max(16, min(int(np.sqrt(rate * target_s)), 1024))
    t = run(side, side)
    return {"value": 2.0 * side * side * k / t / 1e9, "unit": "GFLOP/s", "cores": cores, "kind": "port",
            "sample": f"qgemm {side}x{side}x{k} slice of the 4096^3 workload (reference blocked order, "
                      f"kc=126, OpenMP {cores} threads) in {t:.1f} s"}


def run_reference(args):
    if int(os.environ.get("RANK", "0")) != 0:
        return 0
    if args.warmup > 0:
        cpu_gemm_sample(target_s=2.0)
    vals, base = [], None
    for _ in range(max(args.steps, 1)):
        base = cpu_gemm_sample(target_s=8.0)
        vals.append(base["value"])
    v = round(statistics.median(vals), 6)
    line = {"metric": "qgemm binary128 GFLOP/s (4096^3)", "value": v, "unit": "GFLOP/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "binary128 (host long double / __float128 FMA)", "data": "synthetic (seeded)",
            "config": {"workload": "qgemm m=n=k=4096 row-major NN alpha=1 beta=0, u*2^e entries "
                                   "(sampled m x n slice, full k)"},
            "cpu_baseline": {"value": v, "unit": "GFLOP/s", "cores": base["cores"], "kind": "port",
                             "sample": base["sample"]},
            "e2e": {"value": v, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="qgemm4096", choices=["qgemm4096", "qgemm2048", "qgemm512", "qgemv8192", "qdot26"])
    ap.add_argument("--method", default="ozaki", choices=["softfloat", "ozaki"])
    ap.add_argument("--slices", type=int, default=0)
    ap.add_argument("--bits", type=int, default=0, help="digit width for the Ozaki method (7, 8 or 9)")
    ap.add_argument("--scheme", default="auto", choices=sorted(SCHEMES))
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
    lib = _lib.load()
    pk, pk_src = peaks()
    method = 2 if args.method == "ozaki" else 1
    api.set_method(method)
    slices = args.slices or HEADLINE_DIGITS
    bits = args.bits or HEADLINE_BITS
    api.set_ozaki_slices(slices)
    api.set_ozaki_digit_bits(bits)
    api.set_ozaki_scheme(SCHEMES[args.scheme])

    line = {}
    secondary = {}
    wl = args.workload
    if wl.startswith("qgemm"):
        size = int(wl[5:])
        W = Qgemm(torch, size, size, size, seed=0xC0FFEE + 2 + rank, spread=(size >= 2048))
        # the timed calls record the two events around the tensor-core
        # products only (the roofline's kernel time), so that the other
        # kernels keep overlapping their launches
        lib.quadblas_profile_enable(2 if method == 2 else 0)
        profile_read(lib)
        with ClockSampler(local) as clk:
            ms = time_steps(torch, W.step, args.steps, args.warmup, dist)
        lib.quadblas_profile_enable(0)
        ms_step = ms / args.steps
        value = whole_job_rate(W.flops(), world, ms_step * 1e-3) / 1e9
        if method == 2:
            ph, calls = profile_read(lib)  # warm-up and timed calls, recorded on the launching stream
            tot_calls = max(calls, 1)
            mma_ms = ph[1] / tot_calls
            # every phase: five more calls after the timed region
            lib.quadblas_profile_enable(1)
            for _ in range(5):
                W.step()
            torch.cuda.synchronize()
            lib.quadblas_profile_enable(0)
            phf, callsf = profile_read(lib)
            nf = max(callsf, 1)
            tflops = (ph[3] / tot_calls) / (mma_ms * 1e-3) / 1e12
            # tensor-core products per call, from the profiler's flop count:
            # s(s+1)/2 digit pairs, or one residue product per modulus
            products = int(round(ph[3] / tot_calls / W.flops()))
            crt = products != slices * (slices + 1) // 2 or args.scheme == "residues"
            peak = float(pk.get("bf16_tflops_sustained", FALLBACK["bf16_tflops_sustained"]))
            roof = {"bound": "tensor", "achieved": round(tflops, 1), "peak": peak, "unit": "TFLOP/s",
                    "frac": round(tflops / peak, 4), "traffic": traffic(wl + ("_crt" if crt else ""))[0],
                    "traffic_source": traffic(wl + ("_crt" if crt else ""))[1],
                    "peak_source": pk_src + " (sustained bf16)",
                    "kernel": "ozaki_mma_kernel", "kernel_ms": round(mma_ms, 4),
                    "algorithmic": (f"2*m*n*k*{products} fp16 flops: one product per CRT modulus" if crt else
                                    f"2*m*n*k*{products} flops: s(s+1)/2 digit-pair products"),
                    "phases_ms": {"scale_split": round(phf[0] / nf, 4), "digit_products": round(phf[1] / nf, 4),
                                  "fold": round(phf[2] / nf, 4),
                                  "source": "5 calls after the timed region, with every phase's events"}}
            launches = ozaki_launches(size, slices, bits, crt) * args.steps
            if crt:
                dtype = (f"fp16 residue products modulo {products} moduli in (256, 513] (fp32 accumulate, "
                         "u16 reduced residues, u32-limb CRT reconstruction)")
            else:
                dtype = (f"{'fp16' if bits == 9 else 'bf16'} digit products of {bits}-bit digits "
                         "(fp32 accumulate, int32/192-bit fold)")
        else:
            crt, products = False, None
            roof = {"bound": "int", "achieved": round(W.flops() / (ms_step * 1e-3) / 1e9, 3), "peak": None,
                    "unit": "quad GFLOP/s", "frac": None, "traffic": None,
                    "note": "soft-float kernel is integer-pipe bound"}
            launches = args.steps
            dtype = "u32 (soft-float integer limbs)"
        metric, unit = f"qgemm binary128 GFLOP/s ({size}^3)", "GFLOP/s"
        # the same number of calls as the device-timed headline
        e2e_s, h2d, d2h = W.e2e(max(1, args.steps))
        if dist is not None:
            dist.barrier()
        e2e_s = max_over_ranks(dist, e2e_s)
        if not args.no_secondary and size == 4096:
            pg_s, _, _ = W.e2e(max(1, args.steps), pinned=False)
            pg_s = max_over_ranks(dist, pg_s)
            secondary["e2e_pageable"] = {"value": round(whole_job_rate(W.flops(), world, pg_s) / 1e9, 3),
                                         "unit": unit, "ms_per_step": round(pg_s * 1e3, 3),
                                         "host_buffers": "pageable (not registered with CUDA)"}
        e2e = {"value": round(whole_job_rate(W.flops(), world, e2e_s) / 1e9, 3), "unit": unit,
               "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h)}
        cfg = {"workload": (f"qgemm m=n=k={size} row-major NN alpha=1 beta=0, entries u*2^e (u uniform [-1,1) "
                            "full 113-bit significand, e uniform [-20,20])") if size >= 2048 else
               f"qgemm m=n=k={size} row-major NN alpha=1 beta=0, full-mantissa uniform [-1,1)",
               "method": args.method, "digits_per_operand": slices if method == 2 else None,
               "digit_bits": bits if method == 2 else None,
               "truncation_bits": bits * slices - 1 if method == 2 else None,
               "ozaki_scheme": (("residues (CRT)" if crt else "digit pairs") if method == 2 else None),
               "tensor_products": products if method == 2 else None,
               "l2": "inputs larger than L2 (no flush)" if size >= 2048 else "inputs fit in L2",
               "parallelism": f"replicas x{world}"}

        if not args.no_secondary and size == 4096 and method == 2:
            # soft-float qgemm of the same problem: speed-up and the correctly rounded reference result
            C_oz = to_host(W.dC)
            api.set_method(1)
            ms_sf = time_steps(torch, W.step, 1, 1, dist)
            C_sf = to_host(W.dC)
            sf_gflops = W.flops() / (ms_sf * 1e-3) / 1e9
            secondary["softfloat_qgemm4096"] = {"value": round(sf_gflops, 3), "unit": "GFLOP/s",
                                                "ms_per_step": round(ms_sf, 3),
                                                "ozaki_speedup": round(value / world / sf_gflops, 2)}
            rng = np.random.default_rng(5)
            idx = rng.integers(0, size * size, 4096)
            secondary["ozaki_ulp_vs_exact_oracle"] = oracle_accuracy(W, C_oz, rank)
            d = ulp_distance(C_oz[idx], C_sf[idx])
            secondary["ozaki_ulp_from_correctly_rounded"] = {"max": float(d.max()),
                                                             "max_rel": float(relative_error(C_oz[idx],
                                                                                             C_sf[idx]).max()),
                                                             "exact_frac": float((d == 0).mean()),
                                                             "samples": len(idx),
                                                             "reference": "soft-float GPU qgemm (correctly rounded)"}
            api.set_method(2)
            sweep = []
            lib.quadblas_profile_enable(1)
            for sch, b, s_ in SWEEP:
                try:
                    api.set_ozaki_scheme(SCHEMES[sch])
                    api.set_ozaki_slices(s_)
                    api.set_ozaki_digit_bits(b)
                    profile_read(lib)
                    ms_s = time_steps(torch, W.step, 2, 1, dist) / 2
                except _lib.QblasError as ex:  # a setting this k does not allow
                    sweep.append({"scheme": sch, "digit_bits": b, "digits": s_, "error": str(ex)})
                    continue
                phs, ncalls = profile_read(lib)
                Cs = to_host(W.dC)[idx]
                ds = ulp_distance(Cs, C_sf[idx])
                sweep.append({"scheme": sch, "truncation_bits": b * s_ - 1, "digit_bits": b, "digits": s_,
                              "tensor_products": int(round(phs[3] / max(ncalls, 1) / W.flops())),
                              "ms": round(ms_s, 3), "gflops": round(W.flops() / (ms_s * 1e-3) / 1e9, 1),
                              "speedup_vs_softfloat": round(ms_sf / ms_s, 2),
                              "max_ulp_from_correctly_rounded": float(ds.max()),
                              "max_rel": float(relative_error(Cs, C_sf[idx]).max()),
                              "exact_frac": float((ds == 0).mean())})
            lib.quadblas_profile_enable(0)
            # the library's own default setting (every Ozaki knob at 0)
            api.set_ozaki_scheme(0)
            api.set_ozaki_slices(0)
            api.set_ozaki_digit_bits(0)
            ms_d = time_steps(torch, W.step, args.steps, 1, dist) / args.steps
            C_d = to_host(W.dC)
            dd = ulp_distance(C_d[idx], C_sf[idx])
            secondary["ozaki_library_default"] = {
                "value": round(whole_job_rate(W.flops(), world, ms_d * 1e-3) / 1e9, 3), "unit": "GFLOP/s",
                "ms_per_step": round(ms_d, 4), "setting": "scheme auto, 16 digits of 9 bits (T = 143)",
                "max_ulp_from_correctly_rounded": float(dd.max()), "exact_frac": float((dd == 0).mean()),
                "ulp_vs_exact_oracle": oracle_accuracy(W, C_d, rank, samples=256)}
            api.set_ozaki_scheme(SCHEMES[args.scheme])
            api.set_ozaki_slices(slices)
            api.set_ozaki_digit_bits(bits)
            secondary["ozaki_sweep"] = sweep
        if not args.no_secondary and size == 4096:
            del W
            torch.cuda.empty_cache()
            # qgemv by both methods (identical, correctly rounded results) and qdot
            for name, mk, meth in [("qgemv8192", lambda: Qgemv(torch, 8192, 8192, 11 + rank), 1),
                                   ("qgemv8192_ozaki", lambda: Qgemv(torch, 8192, 8192, 11 + rank), 2),
                                   ("qdot26", lambda: Qdot(torch, 1 << 26, 13 + rank), 1)]:
                api.set_method(meth)
                S = mk()
                ms2 = time_steps(torch, S.step, args.steps, 3, dist) / args.steps
                secondary[name] = {"value": round(S.bytes() / (ms2 * 1e-3) / 1e9, 1), "unit": "GB/s",
                                   "ms_per_step": round(ms2, 4), "method": "ozaki" if meth == 2 else "softfloat",
                                   "roofline": hbm_roofline(pk, pk_src, S.bytes(), ms2, name)}
                del S
                torch.cuda.empty_cache()
            api.set_method(1)
            secondary["batched_config4"] = batched_config4(torch, api, rank)
            # the same batch under the Ozaki method: qgemm problems with m n k >= 2^20 on the
            # grouped residue path (normwise accurate, as their single calls), the rest as above
            api.set_method(2)
            secondary["batched_config4_ozaki"] = batched_config4(torch, api, rank)
            api.set_method(1)
            S = Qgemm(torch, 512, 512, 512, seed=0xC0FFEE, spread=False)
            ms2 = time_steps(torch, S.step, 20, 3, dist) / 20
            secondary["qgemm512_softfloat"] = {"value": round(S.flops() / (ms2 * 1e-3) / 1e9, 3),
                                               "unit": "GFLOP/s", "ms_per_step": round(ms2, 4)}
            api.set_method(method)
    elif wl == "qgemv8192":
        W = Qgemv(torch, 8192, 8192, seed=11 + rank)
        with ClockSampler(local) as clk:
            ms = time_steps(torch, W.step, args.steps, args.warmup, dist)
        ms_step = ms / args.steps
        value = whole_job_rate(W.bytes(), world, ms_step * 1e-3) / 1e9
        metric, unit = "qgemv binary128 GB/s (8192^2 row-major)", "GB/s"
        # soft-float: x unpack, thread-per-row kernel, chunk merge, exact pass;
        # Ozaki: x digits, split + tensor-core kernel, row finish, exact pass
        # (the exact pass returns at once when every row was certified)
        launches = 4 * args.steps
        roof = hbm_roofline(pk, pk_src, W.bytes(), ms_step, wl + ("_ozaki" if method == 2 else ""))
        e2e = None
        dtype = ("fp16 digits x fp16 digits -> fp32 on tcgen05, u32 integer limbs" if method == 2
                 else "u32 (soft-float integer limbs)")
        cfg = {"workload": "qgemv 8192x8192 row-major alpha=1 beta=0, wide-exponent values",
               "method": args.method, "l2": "inputs larger than L2 (no flush)"}
    else:
        W = Qdot(torch, 1 << 26, seed=13 + rank)
        with ClockSampler(local) as clk:
            ms = time_steps(torch, W.step, args.steps, args.warmup, dist)
        ms_step = ms / args.steps
        value = whole_job_rate(W.bytes(), world, ms_step * 1e-3) / 1e9
        metric, unit = "qdot binary128 GB/s (n=2^26)", "GB/s"
        launches = 3 * args.steps  # partial kernel, finalize, exact pass (returns at once)
        roof = hbm_roofline(pk, pk_src, W.bytes(), ms_step, wl)
        e2e, dtype = None, "u32 (soft-float integer limbs)"
        cfg = {"workload": "qdot n=2^26 wide-exponent values with cancelling pairs",
               "l2": "inputs larger than L2 (no flush)"}

    cpu = None
    if rank == 0 and not args.no_cpu and wl == "qgemm4096":
        cpu = cpu_gemm_sample()
        cpu["value"] = round(cpu["value"], 6)

    if rank == 0:
        line = {"metric": metric, "value": round(value, 3), "unit": unit, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(ms_step, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic (seeded)",
                "config": cfg, "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
                "clocks": clk.summary(), "gpu_launches": launches}
        if "ozaki_ulp_vs_exact_oracle" in secondary:
            line["ozaki_ulp_vs_exact_oracle"] = secondary["ozaki_ulp_vs_exact_oracle"]
        if secondary:
            line["secondary"] = secondary
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
