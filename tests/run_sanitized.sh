#!/usr/bin/env bash
# The CPU test suite with the host code under AddressSanitizer and
# UndefinedBehaviorSanitizer: libquadblas_gpu.so's host paths (capi.cpp and
# the host side of every .cu file), the oracle (oracle/oracle.cpp) and the
# device soft-float core compiled as host C++ (tests/softquad_host.cpp) are
# rebuilt into _build_san/ directories with -fsanitize=address,undefined and
# loaded into an uninstrumented Python with the sanitizer runtimes preloaded.
# Any UndefinedBehaviorSanitizer report aborts the test process
# (-fno-sanitize-recover); leak checking is off (the interpreter's own
# allocations are not freed at exit).  Extra arguments go to pytest.
set -euo pipefail
cd "$(dirname "$0")/.."
export QBLAS_SANITIZE=1
ASAN_RT=$(g++ -print-file-name=libasan.so)
UBSAN_RT=$(g++ -print-file-name=libubsan.so)
python -c "from qblas_gb300 import build; build.build()"
python -c "from oracle import oracle; oracle.build()"
export ASAN_OPTIONS=detect_leaks=0:halt_on_error=1:abort_on_error=1
export UBSAN_OPTIONS=print_stacktrace=1:halt_on_error=1
LD_PRELOAD="$ASAN_RT:$UBSAN_RT" python -m pytest tests -x -q -m "not gpu" -p no:cacheprovider "$@"
