"""qblas_gb300: IEEE binary128 BLAS (QuadBLAS's qdot / qgemv / qgemm hot
path) as hand-written CUDA kernels for GB300 (sm_103a), behind the
reference's C ABI (libquadblas_gpu.so, include/quadblas_gpu.h)."""
from . import gen, quad  # noqa: F401

__all__ = ["gen", "quad"]
