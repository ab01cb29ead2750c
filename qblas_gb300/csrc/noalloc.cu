// quadblas_qdot_dev_noalloc: the device-pointer qdot for callers that must
// not allocate device memory.
//
// quadblas_qdot_dev takes its scratch (one partial accumulator per block of
// the first qdot kernel) from the library's stream-ordered memory pool
// (cudaMallocFromPoolAsync).
// Some callers cannot let a library do that: programs that hand all device
// memory to their own allocator or memory plan up front (so a cudaMalloc from
// a library would fail or fragment their pool), and latency-sensitive loops
// that cannot afford a trip into the CUDA allocator or the device-wide
// synchronisation that cudaFree implies.  This entry point runs the same
// qdot kernels, with the same grid, but its scratch is the file-scope array
// below, so it allocates nothing.
//
// The array holds kNoallocPartials = QBLAS_NOALLOC_MAX_PARTIALS accumulators
// (40 bytes each, 40 KiB) followed by the state of the exact pass (16 KiB of
// Kulisch digits); every GPU on which the library's module is loaded keeps it
// until the process exits.  A call needs one accumulator
// per block, min(ceil(n / 1024), 4 x SM count): any n fits on GPUs with up to
// 256 SMs (GB300 has 152); on a larger GPU an n whose block count would exceed
// the array is rejected with QBLAS_ERR_INVALID_VALUE before anything runs.
//
// All calls share the one array and it keeps the last call's contents.
// Nothing in it has to start at zero: every block overwrites its own entry
// before the second kernel reads it, and the second kernel resets the exact
// pass's state whenever it arms that pass.  Calls whose kernels overlap on the GPU
// (the same device, different streams without ordering between them) race on
// the array and may return wrong results; order them on one stream or with
// events.
//
// Set-up: the first call on each device looks up the device address of the
// array (cudaGetSymbolAddress with that device current) and caches it; make
// that first call before any stream capture on that device.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "kernels.h"
#include "quadblas_gpu.h"
#include "exact.cuh"
#include "wacc.cuh"

constexpr int kNoallocPartials = QBLAS_NOALLOC_MAX_PARTIALS;
constexpr size_t kNoallocBytes =
    ((size_t)kNoallocPartials * sizeof(qb::wacc) + 255) / 256 * 256 + sizeof(qb::ExactGlobal);

static __device__ __align__(256) unsigned char g_qdot_noalloc_partials[kNoallocBytes];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void* g_partials_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array on device `dev` (current), looked up once.
int partials_address(int dev, void** out) {
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_partials_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_qdot_noalloc_partials);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      return QBLAS_ERR_CUDA;
    }
    g_partials_addr[dev] = p;
  }
  *out = g_partials_addr[dev];
  return QBLAS_OK;
}

}  // namespace

extern "C" __attribute__((visibility("default"))) int quadblas_qdot_dev_noalloc(
    int64_t n, const void* dx, int64_t incx, const void* dy, int64_t incy, void* d_result,
    void* stream) {
  if (n < 0 || (n > 0 && (incx <= 0 || incy <= 0)) || d_result == nullptr)
    return QBLAS_ERR_INVALID_VALUE;
  if ((((uintptr_t)dx) | ((uintptr_t)dy) | ((uintptr_t)d_result)) & 15u) return QBLAS_ERR_MISALIGNED;
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? QBLAS_ERR_NO_DEVICE
                                                                        : QBLAS_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) return QBLAS_ERR_NO_DEVICE;
  if (qb::dot_scratch_bytes(n) > sizeof(g_qdot_noalloc_partials)) return QBLAS_ERR_INVALID_VALUE;
  void* partials = nullptr;
  int rc = partials_address(dev, &partials);
  if (rc != QBLAS_OK) return rc;
  e = qb::launch_dot(n, static_cast<const qb::q128*>(dx), incx, static_cast<const qb::q128*>(dy),
                     incy, static_cast<qb::q128*>(d_result), 0, partials,
                     static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? QBLAS_OK : QBLAS_ERR_CUDA;
}
