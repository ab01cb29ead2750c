// C ABI of libquadblas_gpu.so (declared in include/quadblas_gpu.h).
//
// The nine reference entry points keep the exact signatures of
// include/quadblas/interface/c_interface.hpp:21-144 (host Sleef_quad
// pointers, double scalars, void/double returns).  Each one stages its
// operands into device buffers owned by this library, runs the kernels on
// an internal stream of the current device and copies the result back
// before returning, so it is a drop-in for the reference's synchronous CPU
// call.  Extensions:
//   *_q   : host pointers, binary128 scalars and results, int64 sizes,
//           status return;
//   *_dev : device pointers on a caller-given CUDA stream (no host sync).
// There is no CPU fallback: with no usable GPU every call fails with
// QBLAS_ERR_NO_DEVICE (reference-compatible calls then return 0 / leave
// outputs unchanged and record the error for quadblas_last_error()).
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <thread>

#include "kernels.h"
#include "quadblas_gpu.h"

using qb::q128;

namespace {

thread_local int g_last_error = 0;
std::atomic<int> g_num_threads{0};
std::atomic<int> g_method{0};   // 0 auto, 1 soft-float, 2 Ozaki
std::atomic<int> g_slices{0};   // 0 = automatic
std::atomic<int> g_ozaki_scheme{0};  // 0 = automatic (residues when they fit), 1 digit pairs, 2 residues
std::atomic<int> g_digit_bits{0};  // 0 = automatic (8)

int fail(int code) {
  g_last_error = code;
  return code;
}

std::atomic<int> g_fail_allocs{0};  // injected allocation failures still to happen

bool take_injected_failure() {
  int v = g_fail_allocs.load();
  while (v > 0)
    if (g_fail_allocs.compare_exchange_weak(v, v - 1)) return true;
  return false;
}

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return qb::kOk;
  // QBLAS_DEBUG set: name the CUDA error behind a failing status on stderr
  static const bool debug = getenv("QBLAS_DEBUG") != nullptr;
  if (debug) fprintf(stderr, "qblas: CUDA error %d: %s\n", (int)e, cudaGetErrorString(e));
  if (e == cudaErrorMemoryAllocation) return qb::kErrNoMemory;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return qb::kErrNoDevice;
  return qb::kErrCuda;
}

q128 q_from_double(double d) {
  uint64_t b;
  memcpy(&b, &d, 8);
  return qb::q_from_double_bits(b);
}

double q_to_double(q128 q) {
  uint64_t b = qb::q_to_double_bits(q);
  double d;
  memcpy(&d, &b, 8);
  return d;
}

q128 q_load(const void* p) {
  q128 v;
  memcpy(&v, p, 16);
  return v;
}

// ---- per-device state for the host-pointer entry points -------------------
enum Slot { kSlotA, kSlotB, kSlotC, kSlotScratch, kSlotResult, kNumSlots };
enum Side { kSideB, kSideC, kSideACopy, kSideA, kNumSides };
enum Event { kEvBDone, kEvCReady, kEvBCopied, kEvACopied, kEvADone, kEvFoldBand, kNumEvents };

struct DevState {
  std::mutex mu;
  cudaStream_t stream = nullptr;
  // host-pointer qgemm (Ozaki): side streams (kSideB: copy and digits of B;
  // kSideC: copies of C in and out; kSideACopy: copies of A's row bands;
  // kSideA: digits of A) and the events that order them
  cudaStream_t side[kNumSides] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t ev[kNumEvents] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  void* buf[kNumSlots] = {nullptr};
  size_t cap[kNumSlots] = {0};
  int* err_host = nullptr;  // pinned: the last host-pointer Ozaki call's error word
};

constexpr int kMaxDevices = 64;
DevState g_dev[kMaxDevices];

int current_device(int& dev) {
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e);
  if (dev < 0 || dev >= kMaxDevices) return qb::kErrNoDevice;
  return qb::kOk;
}

// Per-device timeout flag of device-pointer calls: mapped pinned host
// memory that the Ozaki fold kernel sets (quadblas_device_status reads it).
struct TimeoutFlag {
  std::mutex mu;
  int* host = nullptr;
  int* dev = nullptr;
};
TimeoutFlag g_timeout[kMaxDevices];

int* device_timeout_flag(int dev) {
  if (dev < 0 || dev >= kMaxDevices) return nullptr;
  TimeoutFlag& f = g_timeout[dev];
  std::lock_guard<std::mutex> l(f.mu);
  if (!f.dev) {
    void* h = nullptr;
    if (cudaHostAlloc(&h, sizeof(int), cudaHostAllocMapped) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    void* d = nullptr;
    if (cudaHostGetDevicePointer(&d, h, 0) != cudaSuccess) {
      cudaGetLastError();
      cudaFreeHost(h);
      return nullptr;
    }
    *static_cast<volatile int*>(h) = 0;
    f.host = static_cast<int*>(h);
    f.dev = static_cast<int*>(d);
  }
  return f.dev;
}

int ensure_slot(DevState& st, Slot s, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (st.cap[s] >= bytes) return qb::kOk;
  if (st.buf[s]) {
    cudaStreamSynchronize(st.stream);
    cudaFree(st.buf[s]);
    st.buf[s] = nullptr;
    st.cap[s] = 0;
  }
  size_t want = bytes + bytes / 8;
  cudaError_t e = qb::dev_malloc(&st.buf[s], want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    st.buf[s] = nullptr;
    return cuda_status(e);
  }
  st.cap[s] = want;
  return qb::kOk;
}

// Locks the current device's state and makes sure its stream exists.
struct HostCall {
  DevState* st = nullptr;
  std::unique_lock<std::mutex> lock;
  int status = qb::kOk;
  HostCall() {
    int dev;
    status = current_device(dev);
    if (status) return;
    st = &g_dev[dev];
    lock = std::unique_lock<std::mutex>(st->mu);
    if (!st->stream) {
      cudaError_t e = cudaStreamCreateWithFlags(&st->stream, cudaStreamNonBlocking);
      if (e != cudaSuccess) {
        cudaGetLastError();
        status = cuda_status(e);
      }
    }
  }
};

int ensure_side_streams(DevState& st) {
  for (int i = 0; i < kNumSides; ++i) {
    if (!st.side[i]) {
      cudaError_t e = cudaStreamCreateWithFlags(&st.side[i], cudaStreamNonBlocking);
      if (e != cudaSuccess) {
        cudaGetLastError();
        st.side[i] = nullptr;
        return cuda_status(e);
      }
    }
  }
  for (int i = 0; i < kNumEvents; ++i) {
    if (!st.ev[i]) {
      cudaError_t e = cudaEventCreateWithFlags(&st.ev[i], cudaEventDisableTiming);
      if (e != cudaSuccess) {
        cudaGetLastError();
        st.ev[i] = nullptr;
        return cuda_status(e);
      }
    }
  }
  return qb::kOk;
}

int64_t extent(int64_t rows, int64_t cols, int64_t srow, int64_t scol) {
  if (rows <= 0 || cols <= 0) return 0;
  return (rows - 1) * srow + (cols - 1) * scol + 1;
}

bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

int h2d(void* dst, const void* src, int64_t elems, cudaStream_t s) {
  if (elems <= 0) return qb::kOk;
  return cuda_status(cudaMemcpyAsync(dst, src, (size_t)elems * 16, cudaMemcpyHostToDevice, s));
}
int d2h(void* dst, const void* src, int64_t elems, cudaStream_t s) {
  if (elems <= 0) return qb::kOk;
  return cuda_status(cudaMemcpyAsync(dst, src, (size_t)elems * 16, cudaMemcpyDeviceToHost, s));
}

bool is_trans(char t) { return t == 'T' || t == 't' || t == 'C' || t == 'c'; }
bool is_col(char layout) { return layout == 'C' || layout == 'c'; }

// ---- argument resolution (shared by host and device entry points) --------
struct GemvPlan {
  int64_t m, n;  // op(A) is m x n after the reference's trans handling
  qb::MatView A;
  int64_t a_rows, a_cols;  // storage extent in (row, col) of the view
};

// Reference semantics (c_interface.hpp:76-85): trans swaps m and n and
// flips the layout; then row-major reads A[i*lda + j], column-major
// A[j*lda + i] (level2.hpp:33-44, :72-79).
int plan_gemv(char layout, char trans, int64_t m, int64_t n, int64_t lda, GemvPlan& p) {
  if (m < 0 || n < 0) return qb::kErrInvalidValue;
  bool col = is_col(layout);
  if (is_trans(trans)) {
    std::swap(m, n);
    col = !col;
  }
  p.m = m;
  p.n = n;
  if (!col) {
    if (lda < std::max<int64_t>(1, n)) return qb::kErrInvalidValue;
    p.A.si = lda;
    p.A.sj = 1;
  } else {
    if (lda < std::max<int64_t>(1, m)) return qb::kErrInvalidValue;
    p.A.si = 1;
    p.A.sj = lda;
  }
  p.A.p = nullptr;
  return qb::kOk;
}

struct GemmPlan {
  qb::GemmArgs g;
  int64_t extA, extB, extC;
};

int plan_gemm(char layout, char transa, char transb, int64_t m, int64_t n, int64_t k, int64_t lda,
              int64_t ldb, int64_t ldc, GemmPlan& p) {
  if (m < 0 || n < 0 || k < 0) return qb::kErrInvalidValue;
  bool col = is_col(layout), ta = is_trans(transa), tb = is_trans(transb);
  qb::GemmArgs& g = p.g;
  g.m = m;
  g.n = n;
  g.k = k;
  // op(A) is m x k, op(B) is k x n, C is m x n.
  // Stored A has (ar x ac) = ta ? (k x m) : (m x k); likewise B.
  int64_t ar = ta ? k : m, ac = ta ? m : k;
  int64_t br = tb ? n : k, bc = tb ? k : n;
  if (!col) {
    if (lda < std::max<int64_t>(1, ac) || ldb < std::max<int64_t>(1, bc) ||
        ldc < std::max<int64_t>(1, n))
      return qb::kErrInvalidValue;
    // stored element (r, c) at r*ld + c
    g.sai = ta ? 1 : lda;
    g.sal = ta ? lda : 1;
    g.sbl = tb ? 1 : ldb;
    g.sbj = tb ? ldb : 1;
    g.sci = ldc;
    g.scj = 1;
  } else {
    if (lda < std::max<int64_t>(1, ar) || ldb < std::max<int64_t>(1, br) ||
        ldc < std::max<int64_t>(1, m))
      return qb::kErrInvalidValue;
    // stored element (r, c) at c*ld + r
    g.sai = ta ? lda : 1;
    g.sal = ta ? 1 : lda;
    g.sbl = tb ? ldb : 1;
    g.sbj = tb ? 1 : ldb;
    g.sci = 1;
    g.scj = ldc;
  }
  p.extA = extent(m, k, g.sai, g.sal);
  p.extB = extent(k, n, g.sbl, g.sbj);
  p.extC = extent(m, n, g.sci, g.scj);
  return qb::kOk;
}

// ---- device-pointer implementations -----------------------------------
int dev_dot(int64_t n, const void* dx, int64_t incx, const void* dy, int64_t incy, void* dres,
            int take_sqrt, cudaStream_t s, void* scratch_or_null) {
  if (n < 0 || (n > 0 && (incx <= 0 || incy <= 0))) return qb::kErrInvalidValue;
  if (!aligned16(dx) || !aligned16(dy) || !aligned16(dres)) return qb::kErrMisaligned;
  size_t sb = qb::dot_scratch_bytes(n);
  void* scratch = scratch_or_null;
  if (!scratch && n > 0) {
    cudaError_t e = qb::dev_malloc_async(&scratch, sb, s);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return cuda_status(e);
    }
  }
  cudaError_t e = qb::launch_dot(n, (const q128*)dx, incx, (const q128*)dy, incy, (q128*)dres,
                                 take_sqrt, scratch, s);
  if (!scratch_or_null && scratch) cudaFreeAsync(scratch, s);
  return cuda_status(e);
}

// qgemv method: quadblas_set_method() (1 soft-float, 2 Ozaki), else the
// library's choice by size; every method returns the correctly rounded sums.
int gemv_method() { return g_method.load(); }

int dev_gemv(const GemvPlan& p0, const void* alpha, const void* dA, const void* dx, int64_t incx,
             const void* beta, void* dy, int64_t incy, cudaStream_t s, void* scratch_or_null) {
  GemvPlan p = p0;
  if (p.m > 0 && p.n > 0 && (incx <= 0 || incy <= 0)) return qb::kErrInvalidValue;
  if (!aligned16(dA) || !aligned16(dx) || !aligned16(dy)) return qb::kErrMisaligned;
  p.A.p = (const q128*)dA;
  const int method = gemv_method();
  size_t sb = qb::gemv_scratch_bytes(p.m, p.n, p.A, method);
  void* scratch = scratch_or_null;
  if (!scratch && sb) {
    cudaError_t e = qb::dev_malloc_async(&scratch, sb, s);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return cuda_status(e);
    }
  }
  cudaError_t e = qb::launch_gemv(p.m, p.n, q_load(alpha), p.A, (const q128*)dx, incx, q_load(beta),
                                  (q128*)dy, incy, scratch, s, method);
  if (!scratch_or_null && scratch) cudaFreeAsync(scratch, s);
  return cuda_status(e);
}

// qgemm method: quadblas_set_method(), else the QBLAS_METHOD environment
// variable ("softfloat" / "ozaki"), else automatic (soft-float, which is
// correctly rounded; Ozaki accuracy depends on the digit count).
int gemm_method() {
  int m = g_method.load();
  if (m != 0) return m;
  // read once (a function-local static is initialised once, thread-safely)
  static const int env = [] {
    const char* v = getenv("QBLAS_METHOD");
    return (v && (strcmp(v, "ozaki") == 0 || strcmp(v, "2") == 0)) ? 2 : 1;
  }();
  return env;
}

int gemm_digit_bits() {
  int b = g_digit_bits.load();
  return b ? b : qb::ozaki_default_digit_bits();
}

// Digit count for inner dimension k: the configured count (set_ozaki_slices,
// else QBLAS_SLICES, else the default), capped where the 192-bit fold could
// overflow for this k.
int gemm_digits(int64_t k) {
  int b = gemm_digit_bits();
  int smax = qb::ozaki_digit_cap(b, k);
  int s = g_slices.load();
  if (s > 0) return std::min(s, smax);
  static const int env = [] {
    const char* v = getenv("QBLAS_SLICES");
    const int e = v ? atoi(v) : 0;
    return (e < 2 || e > 22) ? 0 : e;
  }();
  return std::min(env ? env : qb::ozaki_default_digits(b), smax);
}

size_t gemm_scratch_bytes(const GemmPlan& p, int method) {
  if (method != 2) return 0;
  return qb::ozaki_scratch_bytes(p.g.m, p.g.n, p.g.k, gemm_digits(p.g.k), gemm_digit_bits(), g_ozaki_scheme.load());
}

// report: a device-accessible word the fold sets on a timed-out wait, or
// nullptr (the caller checks the call's own error word instead).
int dev_gemm(GemmPlan p, int method, const void* alpha, const void* dA, const void* dB,
             const void* beta, void* dC, cudaStream_t s, void* scratch_or_null,
             const qb::OzakiOverlap* overlap = nullptr, int* report = nullptr) {
  if (!aligned16(dA) || !aligned16(dB) || !aligned16(dC)) return qb::kErrMisaligned;
  p.g.A = (const q128*)dA;
  p.g.B = (const q128*)dB;
  p.g.C = (q128*)dC;
  p.g.alpha = q_load(alpha);
  p.g.beta = q_load(beta);
  if (method != 2) return cuda_status(qb::launch_gemm_softfloat(p.g, s));
  size_t sb = gemm_scratch_bytes(p, method);
  void* scratch = scratch_or_null;
  if (!scratch) {
    cudaError_t e = qb::dev_malloc_async(&scratch, sb, s);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return cuda_status(e);
    }
  }
  cudaError_t e = qb::launch_gemm_ozaki(p.g, gemm_digits(p.g.k), gemm_digit_bits(), scratch, s, overlap,
                                        g_ozaki_scheme.load(), report);
  if (!scratch_or_null) cudaFreeAsync(scratch, s);
  return cuda_status(e);
}

// ---- host-pointer implementations --------------------------------------
int host_dot(int64_t n, const void* x, int64_t incx, const void* y, int64_t incy, void* result,
             int take_sqrt) {
  if (n < 0 || (n > 0 && (incx <= 0 || incy <= 0))) return qb::kErrInvalidValue;
  if (!result || (n > 0 && (!x || !y))) return qb::kErrInvalidValue;
  HostCall hc;
  if (hc.status) return hc.status;
  DevState& st = *hc.st;
  int64_t ex = extent(n, 1, incx, 1), ey = extent(n, 1, incy, 1);
  int rc;
  if ((rc = ensure_slot(st, kSlotA, ex * 16)) || (rc = ensure_slot(st, kSlotB, ey * 16)) ||
      (rc = ensure_slot(st, kSlotResult, 16)) ||
      (rc = ensure_slot(st, kSlotScratch, qb::dot_scratch_bytes(n))))
    return rc;
  if ((rc = h2d(st.buf[kSlotA], x, ex, st.stream)) || (rc = h2d(st.buf[kSlotB], y, ey, st.stream)))
    return rc;
  rc = dev_dot(n, st.buf[kSlotA], incx, st.buf[kSlotB], incy, st.buf[kSlotResult], take_sqrt,
               st.stream, st.buf[kSlotScratch]);
  if (rc) return rc;
  if ((rc = d2h(result, st.buf[kSlotResult], 1, st.stream))) return rc;
  return cuda_status(cudaStreamSynchronize(st.stream));
}

int host_axpy(int64_t n, const void* alpha, const void* x, int64_t incx, void* y, int64_t incy) {
  if (n <= 0) return qb::kOk;  // c_interface.hpp:49
  if (incx <= 0 || incy <= 0 || !x || !y || !alpha) return qb::kErrInvalidValue;
  HostCall hc;
  if (hc.status) return hc.status;
  DevState& st = *hc.st;
  int64_t ex = extent(n, 1, incx, 1), ey = extent(n, 1, incy, 1);
  int rc;
  if ((rc = ensure_slot(st, kSlotA, ex * 16)) || (rc = ensure_slot(st, kSlotC, ey * 16))) return rc;
  if ((rc = h2d(st.buf[kSlotA], x, ex, st.stream)) || (rc = h2d(st.buf[kSlotC], y, ey, st.stream)))
    return rc;
  rc = cuda_status(qb::launch_axpy(n, q_load(alpha), (const q128*)st.buf[kSlotA], incx,
                                   (q128*)st.buf[kSlotC], incy, st.stream));
  if (rc) return rc;
  if ((rc = d2h(y, st.buf[kSlotC], ey, st.stream))) return rc;
  return cuda_status(cudaStreamSynchronize(st.stream));
}

int host_gemv(char layout, char trans, int64_t m, int64_t n, const void* alpha, const void* A,
              int64_t lda, const void* x, int64_t incx, const void* beta, void* y, int64_t incy) {
  GemvPlan p;
  int rc = plan_gemv(layout, trans, m, n, lda, p);
  if (rc) return rc;
  if (p.m == 0 || p.n == 0) return qb::kOk;  // level2.hpp:21,61
  if (incx <= 0 || incy <= 0 || !A || !x || !y || !alpha || !beta) return qb::kErrInvalidValue;
  HostCall hc;
  if (hc.status) return hc.status;
  DevState& st = *hc.st;
  int64_t eA = extent(p.m, p.n, p.A.si, p.A.sj), ex = extent(p.n, 1, incx, 1),
          ey = extent(p.m, 1, incy, 1);
  if ((rc = ensure_slot(st, kSlotA, eA * 16)) || (rc = ensure_slot(st, kSlotB, ex * 16)) ||
      (rc = ensure_slot(st, kSlotC, ey * 16)))
    return rc;
  qb::MatView probe = p.A;
  size_t sb = qb::gemv_scratch_bytes(p.m, p.n, probe, gemv_method());
  if ((rc = ensure_slot(st, kSlotScratch, sb))) return rc;
  if ((rc = h2d(st.buf[kSlotA], A, eA, st.stream)) || (rc = h2d(st.buf[kSlotB], x, ex, st.stream)) ||
      (rc = h2d(st.buf[kSlotC], y, ey, st.stream)))
    return rc;
  rc = dev_gemv(p, alpha, st.buf[kSlotA], st.buf[kSlotB], incx, beta, st.buf[kSlotC], incy, st.stream,
                st.buf[kSlotScratch]);
  if (rc) return rc;
  if ((rc = d2h(y, st.buf[kSlotC], ey, st.stream))) return rc;
  return cuda_status(cudaStreamSynchronize(st.stream));
}

// True when p is in page-locked (pinned or registered) host memory.
bool host_page_locked(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// Copies rows [i0, i1) of the staged C back to the caller once the fold of
// that band (enqueued on the main stream) is done, on side[1].
struct BandCopy {
  DevState* st;
  void* host_C;
  GemmPlan p;
  int64_t copied_rows;
  static int done(void* ctx, int64_t i0, int64_t i1) {
    BandCopy* b = static_cast<BandCopy*>(ctx);
    DevState& s = *b->st;
    const int64_t sci = b->p.g.sci, n = b->p.g.n;
    const int64_t off = i0 * sci, cnt = (i1 - 1 - i0) * sci + n;
    cudaError_t e = cudaEventRecord(s.ev[kEvFoldBand], s.stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s.side[kSideC], s.ev[kEvFoldBand], 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(static_cast<char*>(b->host_C) + off * 16,
                          static_cast<const char*>(s.buf[kSlotC]) + off * 16, (size_t)cnt * 16,
                          cudaMemcpyDeviceToHost, s.side[kSideC]);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return 1;
    }
    b->copied_rows += i1 - i0;
    return 0;
  }
};

// Copies rows [r0, r1) of op(A) into the staged A on kSideACopy, after the
// copy of B (which the first digit products need whole), and makes stream s
// wait for them.  When op(A)'s rows are not contiguous, the first band
// copies all of A.  With c_banded (C's rows contiguous, as the fold's row
// bands need) the same rows of C follow each band of A and c_ready is
// recorded after them; otherwise all of C is queued behind the last band.
struct ARowCopy {
  DevState* st;
  const void* host_A;
  const void* host_C;
  GemmPlan p;
  bool c_banded;
  static int rows(void* ctx, int64_t r0, int64_t r1, cudaStream_t s) {
    ARowCopy* a = static_cast<ARowCopy*>(ctx);
    DevState& d = *a->st;
    const qb::GemmArgs& g = a->p.g;
    cudaStream_t cs = d.side[kSideACopy];
    cudaError_t e = cudaSuccess;
    if (r0 == 0) e = cudaStreamWaitEvent(cs, d.ev[kEvBCopied], 0);
    int64_t off = 0, cnt = 0;
    if (g.sal == 1 && g.sai >= g.k) {
      off = r0 * g.sai;
      cnt = (r1 - 1 - r0) * g.sai + g.k;
    } else if (r0 == 0) {
      cnt = a->p.extA;
    }
    if (e == cudaSuccess && cnt > 0)
      e = cudaMemcpyAsync(static_cast<char*>(d.buf[kSlotA]) + off * 16,
                          static_cast<const char*>(a->host_A) + off * 16, (size_t)cnt * 16,
                          cudaMemcpyHostToDevice, cs);
    if (e == cudaSuccess) e = cudaEventRecord(d.ev[kEvACopied], cs);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, d.ev[kEvACopied], 0);
    if (e == cudaSuccess && a->c_banded) {
      const int64_t coff = r0 * g.sci, ccnt = (r1 - 1 - r0) * g.sci + g.n;
      e = cudaMemcpyAsync(static_cast<char*>(d.buf[kSlotC]) + coff * 16,
                          static_cast<const char*>(a->host_C) + coff * 16, (size_t)ccnt * 16,
                          cudaMemcpyHostToDevice, cs);
      if (e == cudaSuccess) e = cudaEventRecord(d.ev[kEvCReady], cs);
    } else if (e == cudaSuccess && r1 == g.m) {
      cudaStream_t cc = d.side[kSideC];
      e = cudaStreamWaitEvent(cc, d.ev[kEvACopied], 0);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(d.buf[kSlotC], a->host_C, (size_t)a->p.extC * 16, cudaMemcpyHostToDevice, cc);
      if (e == cudaSuccess) e = cudaEventRecord(d.ev[kEvCReady], cc);
    }
    if (e != cudaSuccess) {
      cudaGetLastError();
      return 1;
    }
    return 0;
  }
};

int host_gemm(char layout, char transa, char transb, int64_t m, int64_t n, int64_t k,
              const void* alpha, const void* A, int64_t lda, const void* B, int64_t ldb,
              const void* beta, void* C, int64_t ldc) {
  GemmPlan p;
  int rc = plan_gemm(layout, transa, transb, m, n, k, lda, ldb, ldc, p);
  if (rc) return rc;
  if (m == 0 || n == 0 || k == 0) return qb::kOk;  // level3.hpp:221
  if (!A || !B || !C || !alpha || !beta) return qb::kErrInvalidValue;
  HostCall hc;
  if (hc.status) return hc.status;
  DevState& st = *hc.st;
  const int method = gemm_method();
  if ((rc = ensure_slot(st, kSlotA, p.extA * 16)) || (rc = ensure_slot(st, kSlotB, p.extB * 16)) ||
      (rc = ensure_slot(st, kSlotC, p.extC * 16)) ||
      (rc = ensure_slot(st, kSlotScratch, gemm_scratch_bytes(p, method))))
    return rc;
  if (method == 2 && !st.err_host) {
    void* h = nullptr;
    if (cudaMallocHost(&h, 256) != cudaSuccess) {
      cudaGetLastError();
      return qb::kErrNoMemory;
    }
    st.err_host = static_cast<int*>(h);
  }
  // this call's error word (in its scratch), copied back after the fold and
  // checked once the stream is done; the device-pointer flag is not involved
  auto timed_out = [&]() -> int {
    if (method != 2) return qb::kOk;
    const size_t off = qb::ozaki_error_flag_offset(p.g.m, p.g.n, p.g.k, gemm_digits(p.g.k), gemm_digit_bits(),
                                                   g_ozaki_scheme.load());
    volatile int* h = st.err_host;
    h[0] = h[1] = h[2] = 0;
    return cuda_status(cudaMemcpyAsync(st.err_host, static_cast<char*>(st.buf[kSlotScratch]) + off,
                                       3 * sizeof(int), cudaMemcpyDeviceToHost, st.stream));
  };
  auto check_timeout = [&](int status) -> int {
    if (status || method != 2) return status;
    volatile int* h = st.err_host;
    return (h[0] | h[1] | h[2]) ? qb::kErrTimeout : qb::kOk;
  };
  if (method == 2) {
    // Ozaki, with the host link kept busy in the order the GPU needs the
    // data: B first (copied and cut into digits on kSideB), then A in row
    // bands (each band cut on kSideA as it lands, and the digit products of
    // the tiles that need it start at once), then C (needed by the fold);
    // C comes back band by band on kSideC while later bands fold.
    if ((rc = ensure_side_streams(st))) return rc;
    BandCopy bc{&st, C, p, qb::kOk};
    // C by row bands when its rows are contiguous, the fold goes by row bands
    // and C is page-locked: a copy from or to pageable memory returns only
    // when it is done, so a band copied back before later bands are enqueued
    // would hold the host until that band's fold, and the GPU would wait for it
    const bool c_banded = p.g.scj == 1 && p.g.sci >= p.g.n && p.g.m >= 64 && host_page_locked(C);
    ARowCopy ac{&st, A, C, p, c_banded};
    qb::OzakiOverlap ov{st.side[kSideB],      st.ev[kEvBDone], st.ev[kEvCReady], &BandCopy::done, &bc,
                        &ARowCopy::rows,      &ac,             st.side[kSideA],  st.ev[kEvADone],
                        c_banded ? 1 : 0};
    if ((rc = h2d(st.buf[kSlotB], B, p.extB, st.side[kSideB])) ||
        (rc = cuda_status(cudaEventRecord(st.ev[kEvBCopied], st.side[kSideB]))))
      return rc;
    rc = dev_gemm(p, method, alpha, st.buf[kSlotA], st.buf[kSlotB], beta, st.buf[kSlotC], st.stream,
                  st.buf[kSlotScratch], &ov);
    if (!rc) rc = timed_out();
    if (!rc && bc.copied_rows > 0) {
      // the bands covered C; wait for their copies
      if (bc.copied_rows != p.g.m) rc = qb::kErrCuda;
      int rc2 = cuda_status(cudaStreamSynchronize(st.side[kSideC]));
      int rc3 = cuda_status(cudaStreamSynchronize(st.stream));
      return check_timeout(rc ? rc : (rc2 ? rc2 : rc3));
    }
  } else {
    if ((rc = h2d(st.buf[kSlotA], A, p.extA, st.stream)) ||
        (rc = h2d(st.buf[kSlotB], B, p.extB, st.stream)) ||
        (rc = h2d(st.buf[kSlotC], C, p.extC, st.stream)))
      return rc;
    rc = dev_gemm(p, method, alpha, st.buf[kSlotA], st.buf[kSlotB], beta, st.buf[kSlotC], st.stream,
                  st.buf[kSlotScratch]);
  }
  if (rc) {
    // leave no copy in flight into the staging buffers on any stream
    cudaStreamSynchronize(st.stream);
    for (int i = 0; i < kNumSides; ++i)
      if (st.side[i]) cudaStreamSynchronize(st.side[i]);
    cudaGetLastError();
    return rc;
  }
  if ((rc = d2h(C, st.buf[kSlotC], p.extC, st.stream))) return rc;
  if ((rc = timed_out())) return rc;
  return check_timeout(cuda_status(cudaStreamSynchronize(st.stream)));
}

}  // namespace

namespace qb {
int gemm_method_setting() { return gemm_method(); }
int gemm_digits_setting(int64_t k) { return gemm_digits(k); }
int gemm_bits_setting() { return gemm_digit_bits(); }
int ozaki_scheme_setting() { return g_ozaki_scheme.load(); }

cudaError_t dev_malloc(void** p, size_t bytes) {
  if (take_injected_failure()) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMalloc(p, bytes);
}
// Stream-ordered scratch comes from a memory pool of the library's own per
// device (not the device's default pool, which other code in the process
// may use), created on first use and told to keep freed memory: with the
// default release threshold of 0 a pool hands its memory back at every
// synchronisation and maps it again at the next allocation, which took
// about 0.5 ms per 4096^3 Ozaki qgemm call.  quadblas_release_buffers()
// trims it.
cudaMemPool_t scratch_pool(int dev) {
  static std::mutex mu;
  static cudaMemPool_t pools[64] = {};
  if (dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> l(mu);
  if (!pools[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    uint64_t keep = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    pools[dev] = pool;
  }
  return pools[dev];
}

cudaError_t dev_malloc_async(void** p, size_t bytes, cudaStream_t s) {
  if (take_injected_failure()) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  cudaMemPool_t pool = scratch_pool(dev);
  if (!pool) return cudaMallocAsync(p, bytes, s);
  return cudaMallocFromPoolAsync(p, bytes, pool, s);
}
}  // namespace qb

#define QBLAS_EXPORT extern "C" __attribute__((visibility("default")))

// ===========================================================================
// Reference-compatible entry points (c_interface.hpp:21-144)
// ===========================================================================
QBLAS_EXPORT double quadblas_qdot(int n, void* x, int incx, void* y, int incy) {
  q128 r = qb::q_zero(0);
  int rc = host_dot(n, x, incx, y, incy, &r, 0);
  if (rc) {
    fail(rc);
    return 0.0;
  }
  g_last_error = 0;
  return q_to_double(r);
}

QBLAS_EXPORT double quadblas_qnrm2(int n, void* x, int incx) {
  q128 r = qb::q_zero(0);
  int rc = host_dot(n, x, incx, x, incx, &r, 1);
  if (rc) {
    fail(rc);
    return 0.0;
  }
  g_last_error = 0;
  return q_to_double(r);
}

QBLAS_EXPORT void quadblas_qaxpy(int n, double alpha, void* x, int incx, void* y, int incy) {
  q128 a = q_from_double(alpha);
  int rc = host_axpy(n, &a, x, incx, y, incy);
  g_last_error = rc;
}

QBLAS_EXPORT void quadblas_qgemv(char layout, char trans, int m, int n, double alpha, void* A,
                                 int lda, void* x, int incx, double beta, void* y, int incy) {
  q128 a = q_from_double(alpha), b = q_from_double(beta);
  g_last_error = host_gemv(layout, trans, m, n, &a, A, lda, x, incx, &b, y, incy);
}

QBLAS_EXPORT void quadblas_qgemm(char layout, char transa, char transb, int m, int n, int k,
                                 double alpha, void* A, int lda, void* B, int ldb, double beta,
                                 void* C, int ldc) {
  q128 a = q_from_double(alpha), b = q_from_double(beta);
  g_last_error = host_gemm(layout, transa, transb, m, n, k, &a, A, lda, B, ldb, &b, C, ldc);
}

QBLAS_EXPORT void quadblas_set_num_threads(int num_threads) {
  g_num_threads.store(num_threads > 0 ? num_threads : 0);
}

QBLAS_EXPORT int quadblas_get_num_threads(void) {
  int v = g_num_threads.load();
  if (v > 0) return v;
  unsigned hc = std::thread::hardware_concurrency();
  return hc ? (int)hc : 1;
}

QBLAS_EXPORT const char* quadblas_get_version(void) {
  return "QuadBLAS 1.0.0 - qblas-gb300 binary128 BLAS for sm_103a";
}

QBLAS_EXPORT int quadblas_is_aligned(const void* ptr) {
  return ((uintptr_t)ptr % 32u) == 0;  // core/constants.hpp:18 (ALIGNMENT = 32)
}

// ===========================================================================
// Extensions: binary128 scalars/results on host pointers
// ===========================================================================
QBLAS_EXPORT int quadblas_qdot_q(int64_t n, const void* x, int64_t incx, const void* y,
                                 int64_t incy, void* result) {
  return fail(host_dot(n, x, incx, y, incy, result, 0));
}
QBLAS_EXPORT int quadblas_qnrm2_q(int64_t n, const void* x, int64_t incx, void* result) {
  return fail(host_dot(n, x, incx, x, incx, result, 1));
}
QBLAS_EXPORT int quadblas_qaxpy_q(int64_t n, const void* alpha, const void* x, int64_t incx,
                                  void* y, int64_t incy) {
  return fail(host_axpy(n, alpha, x, incx, y, incy));
}
QBLAS_EXPORT int quadblas_qgemv_q(char layout, char trans, int64_t m, int64_t n, const void* alpha,
                                  const void* A, int64_t lda, const void* x, int64_t incx,
                                  const void* beta, void* y, int64_t incy) {
  return fail(host_gemv(layout, trans, m, n, alpha, A, lda, x, incx, beta, y, incy));
}
QBLAS_EXPORT int quadblas_qgemm_q(char layout, char transa, char transb, int64_t m, int64_t n,
                                  int64_t k, const void* alpha, const void* A, int64_t lda,
                                  const void* B, int64_t ldb, const void* beta, void* C,
                                  int64_t ldc) {
  return fail(host_gemm(layout, transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc));
}

// ===========================================================================
// Extensions: device pointers, stream-ordered (stream is a cudaStream_t)
// ===========================================================================
QBLAS_EXPORT int quadblas_qdot_dev(int64_t n, const void* dx, int64_t incx, const void* dy,
                                   int64_t incy, void* d_result, void* stream) {
  return fail(dev_dot(n, dx, incx, dy, incy, d_result, 0, (cudaStream_t)stream, nullptr));
}
QBLAS_EXPORT int quadblas_qnrm2_dev(int64_t n, const void* dx, int64_t incx, void* d_result,
                                    void* stream) {
  return fail(dev_dot(n, dx, incx, dx, incx, d_result, 1, (cudaStream_t)stream, nullptr));
}
QBLAS_EXPORT int quadblas_qaxpy_dev(int64_t n, const void* alpha, const void* dx, int64_t incx,
                                    void* dy, int64_t incy, void* stream) {
  if (n <= 0) return fail(qb::kOk);
  if (incx <= 0 || incy <= 0 || !alpha) return fail(qb::kErrInvalidValue);
  if (!aligned16(dx) || !aligned16(dy)) return fail(qb::kErrMisaligned);
  return fail(cuda_status(qb::launch_axpy(n, q_load(alpha), (const q128*)dx, incx, (q128*)dy, incy,
                                          (cudaStream_t)stream)));
}
QBLAS_EXPORT int quadblas_qgemv_dev(char layout, char trans, int64_t m, int64_t n,
                                    const void* alpha, const void* dA, int64_t lda, const void* dx,
                                    int64_t incx, const void* beta, void* dy, int64_t incy,
                                    void* stream) {
  GemvPlan p;
  int rc = plan_gemv(layout, trans, m, n, lda, p);
  if (rc) return fail(rc);
  if (p.m == 0 || p.n == 0) return fail(qb::kOk);
  if (!alpha || !beta) return fail(qb::kErrInvalidValue);
  return fail(dev_gemv(p, alpha, dA, dx, incx, beta, dy, incy, (cudaStream_t)stream, nullptr));
}
QBLAS_EXPORT int quadblas_qgemm_dev(char layout, char transa, char transb, int64_t m, int64_t n,
                                    int64_t k, const void* alpha, const void* dA, int64_t lda,
                                    const void* dB, int64_t ldb, const void* beta, void* dC,
                                    int64_t ldc, void* stream) {
  GemmPlan p;
  int rc = plan_gemm(layout, transa, transb, m, n, k, lda, ldb, ldc, p);
  if (rc) return fail(rc);
  if (m == 0 || n == 0 || k == 0) return fail(qb::kOk);
  if (!alpha || !beta) return fail(qb::kErrInvalidValue);
  int dev = 0;
  int* report = cudaGetDevice(&dev) == cudaSuccess ? device_timeout_flag(dev) : nullptr;
  return fail(dev_gemm(p, gemm_method(), alpha, dA, dB, beta, dC, (cudaStream_t)stream, nullptr, nullptr,
                       report));
}

// ===========================================================================
// Batched problems, one call each (the batch's serial baseline)
// ===========================================================================
QBLAS_EXPORT int quadblas_batch_run_serial(const qblas_problem* problems, int64_t count, void* stream) {
  if (count < 0 || (count > 0 && !problems)) return fail(qb::kErrInvalidValue);
  cudaStream_t s = (cudaStream_t)stream;
  for (int64_t i = 0; i < count; ++i) {
    const qblas_problem& q = problems[i];
    int rc = qb::kOk;
    if (q.op == QBLAS_OP_GEMM) {
      GemmPlan p;
      rc = plan_gemm(q.layout, q.transa, q.transb, q.m, q.n, q.k, q.lda, q.ldb, q.ldc, p);
      // soft-float, as the batch, except the problems the batch gives to the
      // grouped residue path
      if (!rc && q.m > 0 && q.n > 0 && q.k > 0)
        rc = dev_gemm(p, qb::batch_gemm_routed(q.m, q.n, q.k) ? 2 : 1, q.alpha, q.A, q.B, q.beta, q.C, s, nullptr);
    } else if (q.op == QBLAS_OP_GEMV) {
      GemvPlan p;
      rc = plan_gemv(q.layout, q.transa, q.m, q.n, q.lda, p);
      if (!rc && p.m > 0 && p.n > 0) rc = dev_gemv(p, q.alpha, q.A, q.B, q.ldb, q.beta, q.C, q.ldc, s, nullptr);
    } else if (q.op == QBLAS_OP_DOT) {
      rc = dev_dot(q.n, q.A, q.lda, q.B, q.ldb, q.C, 0, s, nullptr);
    } else {
      rc = qb::kErrInvalidValue;
    }
    if (rc) return fail(rc);
  }
  return fail(qb::kOk);
}

// ===========================================================================
// Configuration and errors
// ===========================================================================
QBLAS_EXPORT int quadblas_set_method(int method) {
  if (method < 0 || method > 2) return fail(qb::kErrInvalidValue);
  g_method.store(method);
  return fail(qb::kOk);
}
QBLAS_EXPORT int quadblas_get_method(void) { return g_method.load(); }
QBLAS_EXPORT int quadblas_release_buffers(void) {
  int dev = 0;
  int rc = current_device(dev);
  if (rc) return fail(rc);
  DevState& st = g_dev[dev];
  std::lock_guard<std::mutex> l(st.mu);
  if (st.stream) cudaStreamSynchronize(st.stream);
  for (int i = 0; i < kNumSides; ++i)
    if (st.side[i]) cudaStreamSynchronize(st.side[i]);
  for (int i = 0; i < kNumSlots; ++i) {
    if (st.buf[i]) cudaFree(st.buf[i]);
    st.buf[i] = nullptr;
    st.cap[i] = 0;
  }
  // the scratch pool's unused memory (frees still pending in stream order stay)
  if (cudaMemPool_t pool = qb::scratch_pool(dev)) cudaMemPoolTrimTo(pool, 0);
  cudaGetLastError();
  return fail(qb::kOk);
}

QBLAS_EXPORT int quadblas_debug_fail_allocations(int count) {
  if (count < 0) return fail(qb::kErrInvalidValue);
  g_fail_allocs.store(count);
  return fail(qb::kOk);
}

QBLAS_EXPORT int quadblas_debug_stall_next_call(int which) {
  if (which == 1)
    qb::ozaki_debug_stall_next();
  else if (which == 2)
    qb::ozgemv_debug_stall_next();
  else
    return fail(qb::kErrInvalidValue);
  return fail(qb::kOk);
}

static unsigned* g_exact_rows_host = nullptr;

QBLAS_EXPORT int quadblas_debug_count_exact_rows(int on) {
  if (on && !g_exact_rows_host) {
    void* p = nullptr;
    if (cudaMallocHost(&p, sizeof(unsigned)) != cudaSuccess) {
      cudaGetLastError();
      return fail(qb::kErrNoMemory);
    }
    g_exact_rows_host = static_cast<unsigned*>(p);
    *g_exact_rows_host = 0;
  }
  qb::gemv_count_exact_rows(on ? g_exact_rows_host : nullptr);
  return fail(qb::kOk);
}

QBLAS_EXPORT long long quadblas_debug_exact_rows(void) {
  return g_exact_rows_host ? (long long)*reinterpret_cast<volatile unsigned*>(g_exact_rows_host) : -1;
}

QBLAS_EXPORT int quadblas_set_ozaki_slices(int slices) {
  if (slices < 0 || slices == 1 || slices > 22) return fail(qb::kErrInvalidValue);
  g_slices.store(slices);
  return fail(qb::kOk);
}
QBLAS_EXPORT int quadblas_get_ozaki_slices(void) { return g_slices.load(); }
QBLAS_EXPORT int quadblas_set_ozaki_digit_bits(int bits) {
  if (bits != 0 && (bits < 7 || bits > 9)) return fail(qb::kErrInvalidValue);
  g_digit_bits.store(bits);
  return fail(qb::kOk);
}
QBLAS_EXPORT int quadblas_get_ozaki_digit_bits(void) { return g_digit_bits.load(); }
QBLAS_EXPORT int quadblas_set_ozaki_scheme(int scheme) {
  if (scheme < 0 || scheme > 2) return fail(qb::kErrInvalidValue);
  g_ozaki_scheme.store(scheme);
  return fail(qb::kOk);
}
QBLAS_EXPORT int quadblas_get_ozaki_scheme(void) { return g_ozaki_scheme.load(); }
QBLAS_EXPORT int quadblas_profile_enable(int on) {
  qb::ozaki_profile_enable(on == 2 ? 2 : (on != 0 ? 1 : 0));
  return qb::kOk;
}
QBLAS_EXPORT int quadblas_profile_read(double* out4, int* calls) {
  if (!out4 || !calls) return fail(qb::kErrInvalidValue);
  return qb::ozaki_profile_read(out4, calls);
}
QBLAS_EXPORT int quadblas_device_status(int clear) {
  int dev = 0;
  int rc = current_device(dev);
  if (rc) return fail(rc);
  TimeoutFlag& f = g_timeout[dev];
  std::lock_guard<std::mutex> l(f.mu);
  if (!f.host) return fail(qb::kOk);  // no device-pointer Ozaki call yet
  volatile int* h = f.host;
  const int set = *h;
  if (clear) *h = 0;
  return fail(set ? qb::kErrTimeout : qb::kOk);
}
QBLAS_EXPORT int quadblas_last_error(void) { return g_last_error; }
QBLAS_EXPORT const char* quadblas_error_string(int code) {
  switch (code) {
    case qb::kOk: return "success";
    case qb::kErrInvalidValue: return "invalid argument";
    case qb::kErrCuda: return "CUDA error";
    case qb::kErrNoMemory: return "out of device memory";
    case qb::kErrNotSupported: return "not supported";
    case qb::kErrNoDevice: return "no usable CUDA device";
    case qb::kErrMisaligned: return "device pointer not 16-byte aligned";
    case qb::kErrTimeout: return "a device-side wait timed out (outputs of that call are NaN)";
    default: return "unknown error";
  }
}
