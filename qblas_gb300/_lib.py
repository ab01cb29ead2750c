"""ctypes binding of libquadblas_gpu.so (the C ABI in include/quadblas_gpu.h).

There is no fallback: if the library is not built, loading fails with an
error telling how to build it."""
from __future__ import annotations

import ctypes
import os

from .build import LIB

_lib = None

i64 = ctypes.c_int64
vp = ctypes.c_void_p
ci = ctypes.c_int
cc = ctypes.c_char
cd = ctypes.c_double

_SIGS = {
    # reference-compatible
    "quadblas_qdot": (cd, [ci, vp, ci, vp, ci]),
    "quadblas_qnrm2": (cd, [ci, vp, ci]),
    "quadblas_qaxpy": (None, [ci, cd, vp, ci, vp, ci]),
    "quadblas_qgemv": (None, [cc, cc, ci, ci, cd, vp, ci, vp, ci, cd, vp, ci]),
    "quadblas_qgemm": (None, [cc, cc, cc, ci, ci, ci, cd, vp, ci, vp, ci, cd, vp, ci]),
    "quadblas_set_num_threads": (None, [ci]),
    "quadblas_get_num_threads": (ci, []),
    "quadblas_get_version": (ctypes.c_char_p, []),
    "quadblas_is_aligned": (ci, [vp]),
    # binary128 host-pointer extensions
    "quadblas_qdot_q": (ci, [i64, vp, i64, vp, i64, vp]),
    "quadblas_qnrm2_q": (ci, [i64, vp, i64, vp]),
    "quadblas_qaxpy_q": (ci, [i64, vp, vp, i64, vp, i64]),
    "quadblas_qgemv_q": (ci, [cc, cc, i64, i64, vp, vp, i64, vp, i64, vp, vp, i64]),
    "quadblas_qgemm_q": (ci, [cc, cc, cc, i64, i64, i64, vp, vp, i64, vp, i64, vp, vp, i64]),
    # device-pointer extensions
    "quadblas_qdot_dev": (ci, [i64, vp, i64, vp, i64, vp, vp]),
    "quadblas_qnrm2_dev": (ci, [i64, vp, i64, vp, vp]),
    "quadblas_qaxpy_dev": (ci, [i64, vp, vp, i64, vp, i64, vp]),
    "quadblas_qgemv_dev": (ci, [cc, cc, i64, i64, vp, vp, i64, vp, i64, vp, vp, i64, vp]),
    "quadblas_qgemm_dev": (ci, [cc, cc, cc, i64, i64, i64, vp, vp, i64, vp, i64, vp, vp, i64, vp]),
    "quadblas_qdot_dev_noalloc": (ci, [i64, vp, i64, vp, i64, vp, vp]),
    # batched
    "quadblas_batch_plan": (ci, [vp, i64, vp]),
    "quadblas_batch_execute": (ci, [vp, vp]),
    "quadblas_batch_destroy": (ci, [vp]),
    "quadblas_batch_info": (ci, [vp, vp]),
    "quadblas_batch_autotune": (ci, [vp]),
    "quadblas_batch_set_grain": (ci, [i64]),
    "quadblas_batch_info_ex": (ci, [vp, vp, i64]),
    "quadblas_batch_setting": (ci, [vp, vp]),
    "quadblas_batch_configure": (ci, [i64, ci]),
    "quadblas_batch_set_ozaki_min": (ci, [i64]),
    "quadblas_batch_run_serial": (ci, [vp, i64, vp]),
    "quadblas_qgemm_batched_dev": (ci, [vp, i64, vp]),
    # configuration
    "quadblas_set_method": (ci, [ci]),
    "quadblas_get_method": (ci, []),
    "quadblas_set_ozaki_slices": (ci, [ci]),
    "quadblas_get_ozaki_slices": (ci, []),
    "quadblas_set_ozaki_digit_bits": (ci, [ci]),
    "quadblas_get_ozaki_digit_bits": (ci, []),
    "quadblas_set_ozaki_scheme": (ci, [ci]),
    "quadblas_get_ozaki_scheme": (ci, []),
    "quadblas_profile_enable": (ci, [ci]),
    "quadblas_profile_read": (ci, [vp, vp]),
    "quadblas_release_buffers": (ci, []),
    "quadblas_debug_fail_allocations": (ci, [ci]),
    "quadblas_debug_stall_next_call": (ci, [ci]),
    "quadblas_debug_count_exact_rows": (ci, [ci]),
    "quadblas_debug_exact_rows": (ctypes.c_longlong, []),
    "quadblas_device_status": (ci, [ci]),
    "quadblas_last_error": (ci, []),
    "quadblas_error_string": (ctypes.c_char_p, [ci]),
}

SYMBOLS = tuple(_SIGS)


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RuntimeError(
                f"{LIB} is not built: run `python -c 'import __graft_entry__ as g; g.build()'` "
                "(or python -m qblas_gb300.build)")
        lib = ctypes.CDLL(LIB)
        for name, (res, args) in _SIGS.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


class QblasError(RuntimeError):
    pass


def check(status: int) -> None:
    if status != 0:
        msg = load().quadblas_error_string(status).decode()
        raise QblasError(f"quadblas error {status}: {msg}")
