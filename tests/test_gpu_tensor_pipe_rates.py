"""Legacy warp-level tensor-core rates on this GPU (tests/tensor_pipe_rates.cu):
mma.sync int8 (m16n8k32, exact int32 sums) and fp16 (m16n8k16, fp32 sums),
the alternatives to the tcgen05 kind::f16 residue products of the Ozaki
qgemm.  The CPU test only compiles the program for sm_103a; the GPU test runs
it, checks the rates are positive and below the nominal dense peaks, and
prints the JSON line."""
import json
import os
import subprocess

import pytest

TESTS = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(TESTS, "tensor_pipe_rates.cu")
EXE = os.path.join(TESTS, "_build", "tensor_pipe_rates")


def _build():
    if not os.path.exists(EXE) or os.path.getmtime(EXE) < os.path.getmtime(SRC):
        os.makedirs(os.path.dirname(EXE), exist_ok=True)
        subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", EXE, SRC], check=True)
    return EXE


def test_tensor_pipe_rates_compiles():
    assert os.access(_build(), os.X_OK)


@pytest.mark.gpu
def test_tensor_pipe_rates_run(torch_cuda):
    out = subprocess.run([_build()], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    r = json.loads(out.stdout.strip().splitlines()[-1])
    print(json.dumps(r))
    assert 0 < r["mma_sync_s8_tops"] < 20000
    assert 0 < r["mma_sync_f16_tflops"] < 5000
