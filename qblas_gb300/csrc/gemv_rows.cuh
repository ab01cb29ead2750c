// The list of qgemv rows whose rounding could not be certified, shared by
// the soft-float and Ozaki qgemv kernels (level2.cu, ozgemv.cu).
#pragma once
#include "exact.cuh"
#include "kernels.h"

namespace qb {

// Every row's rounding is certified (exact.cuh).  Rows that cannot be
// (sums cancelling below the wide accumulator's frame) are left untouched
// and listed in scratch; qgemv_exact_kernel recomputes them exactly and
// returns at once when the list is empty.  (The fast kernels keep no exact
// accumulator in shared memory: the unpacked x is meant to stay in L1.)
struct RowList {
  unsigned count;
  unsigned pad[63];
  int64_t row[1];  // m entries
};

__device__ __forceinline__ void gemv_finish_row(q128 alpha, const wacc& acc, uint64_t err, q128 beta,
                                                q128* yp, int64_t row, RowList* L) {
  q128 r;
  if (wacc_round_certified(acc, err, r))
    *yp = q_epilogue(alpha, r, beta, *yp);
  else
    L->row[atomicAdd(&L->count, 1u)] = row;
}

// Ozaki-split qgemv (ozgemv.cu): y = alpha * op(A) x + beta * y with every
// row certified or listed in `list` for the exact pass of level2.cu.
size_t gemv_ozaki_scratch_bytes(int64_t m, int64_t n);
cudaError_t launch_gemv_ozaki(int64_t m, int64_t n, q128 alpha, MatView A, const q128* x, int64_t incx,
                              q128 beta, q128* y, int64_t incy, RowList* list, void* scratch, cudaStream_t s);

}  // namespace qb
