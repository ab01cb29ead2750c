"""Builds libquadblas_gpu.so in-tree (qblas_gb300/_build/) with nvcc for
sm_103a only.  Translation units are compiled in parallel and linked with
the static CUDA runtime, so the library needs nothing but the driver.

With QBLAS_SANITIZE=1 in the environment the host code is instrumented with
AddressSanitizer and UndefinedBehaviorSanitizer and the library goes to
qblas_gb300/_build_san/ instead (load it with libasan and libubsan preloaded,
as tests/run_sanitized.sh does)."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
SANITIZE = os.environ.get("QBLAS_SANITIZE", "") not in ("", "0")
BUILD = os.path.join(HERE, "_build_san" if SANITIZE else "_build")
LIB = os.path.join(BUILD, "libquadblas_gpu.so")
SAN_FLAGS = ["-Xcompiler", "-fsanitize=address", "-Xcompiler", "-fsanitize=undefined", "-Xcompiler",
             "-fno-omit-frame-pointer", "-Xcompiler", "-fno-sanitize-recover=undefined"]

SOURCES = ["level1.cu", "level2.cu", "level3.cu", "ozaki.cu", "ozgemv.cu", "batched.cu", "noalloc.cu", "capi.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden",
          "-I", CSRC, "-I", os.path.join(ROOT, "include")] + (SAN_FLAGS if SANITIZE else [])


def nvcc() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    for cand in ("/usr/local/cuda/bin/nvcc", "/usr/local/cuda-13.0/bin/nvcc"):
        if os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    if os.path.exists(obj) and os.path.getmtime(obj) > _newest_input(path):
        return obj
    cmd = [nvcc()] + ARCH + COMMON + ["-c", path, "-o", obj]
    if verbose and src.endswith(".cu"):
        cmd += ["-Xptxas", "-v"]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{out.stdout}\n{out.stderr}")
    if verbose and out.stderr:
        sys.stderr.write(out.stderr)
    return obj


def _newest_input(src: str) -> float:
    t = os.path.getmtime(src)
    for f in os.listdir(CSRC):
        if f.endswith((".cuh", ".h")):
            t = max(t, os.path.getmtime(os.path.join(CSRC, f)))
    t = max(t, os.path.getmtime(os.path.join(ROOT, "include", "quadblas_gpu.h")))
    return t


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    newest = max(os.path.getmtime(o) for o in objs)
    if not (os.path.exists(LIB) and os.path.getmtime(LIB) >= newest):
        tmp = LIB + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-cudart", "static"] + (SAN_FLAGS if SANITIZE else [])
        out = subprocess.run(cmd, capture_output=True, text=True)
        if out.returncode != 0:
            raise RuntimeError(f"link failed:\n{out.stdout}\n{out.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
