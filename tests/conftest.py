import os
import subprocess
import sys

import numpy as np
import pytest

TESTS = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(TESTS)
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def O():
    """The oracle (test infrastructure): CPU restatement + exact accumulator."""
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def qlib():
    """libquadblas_gpu.so, built in-tree for sm_103a (cross-compiles without a GPU)."""
    from qblas_gb300 import _lib, build
    build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def sq():
    """The device soft-float core compiled as host C++ (tests/softquad_host.cpp)."""
    import ctypes
    san = os.environ.get("QBLAS_SANITIZE", "") not in ("", "0")
    out = os.path.join(TESTS, "_build_san" if san else "_build", "libsoftquad_host.so")
    src = os.path.join(TESTS, "softquad_host.cpp")
    deps = [src] + [os.path.join(ROOT, "qblas_gb300", "csrc", f) for f in ("softquad.cuh", "wacc.cuh", "exact.cuh", "ozaki.cuh", "ozgemv.cuh", "ozcrt.cuh")]
    if not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(d) for d in deps):
        os.makedirs(os.path.dirname(out), exist_ok=True)
        flags = ["-fsanitize=address,undefined", "-fno-omit-frame-pointer", "-fno-sanitize-recover=undefined"]
        subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-o", out, src] + (flags if san else []),
                       check=True)
    return ctypes.CDLL(out)


@pytest.fixture(scope="session")
def torch_cuda():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return torch


def to_dev(torch, a: np.ndarray):
    a = np.ascontiguousarray(a, dtype=np.uint64)
    return torch.from_numpy(a.view(np.int64)).cuda()


def to_host(t) -> np.ndarray:
    return np.ascontiguousarray(t.cpu().numpy()).view(np.uint64)
