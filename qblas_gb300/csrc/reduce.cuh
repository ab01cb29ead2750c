// Device-side reductions of wide accumulators (warp shuffles, shared
// memory, and the grid-level partials pass).  The merge order is a fixed
// tree, so results are bit-reproducible from run to run.
#pragma once
#include "wacc.cuh"

namespace qb {

__device__ __forceinline__ wacc wacc_shfl_down(const wacc& a, int d) {
  wacc b;
  b.w0 = __shfl_down_sync(0xffffffffu, a.w0, d);
  b.w1 = __shfl_down_sync(0xffffffffu, a.w1, d);
  b.w2 = __shfl_down_sync(0xffffffffu, a.w2, d);
  b.w3 = __shfl_down_sync(0xffffffffu, a.w3, d);
  b.w4 = __shfl_down_sync(0xffffffffu, a.w4, d);
  b.w5 = __shfl_down_sync(0xffffffffu, a.w5, d);
  b.w6 = __shfl_down_sync(0xffffffffu, a.w6, d);
  b.w7 = __shfl_down_sync(0xffffffffu, a.w7, d);
  b.e = __shfl_down_sync(0xffffffffu, a.e, d);
  b.flags = __shfl_down_sync(0xffffffffu, a.flags, d);
  return b;
}

// After the call lane 0 holds the merge of all 32 lanes.
__device__ __forceinline__ void wacc_warp_reduce(wacc& a) {
#pragma unroll
  for (int d = 16; d >= 1; d >>= 1) {
    wacc b = wacc_shfl_down(a, d);
    wacc_merge(a, b);
  }
}

// Block-wide reduction; the result is valid in thread 0.  `sm` must hold
// one wacc per warp.  Contains __syncthreads(): all threads must call it.
__device__ __forceinline__ void wacc_block_reduce(wacc& a, wacc* sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = (blockDim.x + 31) >> 5;
  wacc_warp_reduce(a);
  if (lane == 0) sm[warp] = a;
  __syncthreads();
  if (warp == 0) {
    if (lane < nwarps) {
      a = sm[lane];
    } else {
      wacc_init(a);
    }
    wacc_warp_reduce(a);
  }
  __syncthreads();
}

__device__ __forceinline__ void wacc_store(wacc* p, const wacc& a) { *p = a; }
__device__ __forceinline__ wacc wacc_load(const wacc* p) { return *p; }

// 16-byte streaming load of a binary128 element (evict-first; the data is
// read once).
__device__ __forceinline__ q128 ld_stream(const q128* p) {
  ulonglong2 v = __ldcs(reinterpret_cast<const ulonglong2*>(p));
  q128 r;
  r.lo = v.x;
  r.hi = v.y;
  return r;
}
// 16-byte load through the read-only path (data reused from L1/L2).
__device__ __forceinline__ q128 ld_cached(const q128* p) {
  ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(p));
  q128 r;
  r.lo = v.x;
  r.hi = v.y;
  return r;
}

}  // namespace qb
