// ORACLE — test infrastructure only; never linked into the product.
//
// Builds the reference QuadBLAS itself (its unmodified headers, included
// from the reference tree at build time through the SLEEF shim in
// sleef_shim/) into oracle/_ref/libqref.so.  The wrappers below only give
// the header-only reference a set of exported C symbols with explicit
// OpenMP thread counts, so that tests can run the reference's own code on
// the same inputs as the restatement in oracle.cpp and the GPU kernels.
#include "quadblas/quadblas.hpp"

#include <omp.h>
#include <stdint.h>

using QuadBLAS::Layout;

extern "C" {

void qref_dot(int64_t n, const Sleef_quad* x, int64_t incx, const Sleef_quad* y, int64_t incy,
              int nthreads, Sleef_quad* out) {
  omp_set_num_threads(nthreads);
  *out = QuadBLAS::dot((size_t)n, x, (size_t)incx, y, (size_t)incy);
}

void qref_axpy(int64_t n, const Sleef_quad* alpha, const Sleef_quad* x, int64_t incx,
               Sleef_quad* y, int64_t incy, int nthreads) {
  omp_set_num_threads(nthreads);
  QuadBLAS::axpy((size_t)n, *alpha, x, (size_t)incx, y, (size_t)incy);
}

void qref_gemv(int col_major, int64_t m, int64_t n, const Sleef_quad* alpha, const Sleef_quad* A,
               int64_t lda, const Sleef_quad* x, int64_t incx, const Sleef_quad* beta,
               Sleef_quad* y, int64_t incy, int nthreads) {
  omp_set_num_threads(nthreads);
  QuadBLAS::gemv(col_major ? Layout::ColMajor : Layout::RowMajor, (size_t)m, (size_t)n, *alpha, A,
                 (size_t)lda, x, (size_t)incx, *beta, y, (size_t)incy);
}

void qref_gemm(int col_major, int64_t m, int64_t n, int64_t k, const Sleef_quad* alpha,
               const Sleef_quad* A, int64_t lda, const Sleef_quad* B, int64_t ldb,
               const Sleef_quad* beta, Sleef_quad* C, int64_t ldc, int nthreads) {
  omp_set_num_threads(nthreads);
  QuadBLAS::gemm(col_major ? Layout::ColMajor : Layout::RowMajor, (size_t)m, (size_t)n, (size_t)k,
                 *alpha, A, (size_t)lda, B, (size_t)ldb, *beta, C, (size_t)ldc);
}

// The reference's own C interface entry points (interface/c_interface.hpp),
// re-exported under a prefix because they are declared inline there.
double qref_c_qdot(int n, void* x, int incx, void* y, int incy) {
  return quadblas_qdot(n, x, incx, y, incy);
}
double qref_c_qnrm2(int n, void* x, int incx) { return quadblas_qnrm2(n, x, incx); }
void qref_c_qaxpy(int n, double alpha, void* x, int incx, void* y, int incy) {
  quadblas_qaxpy(n, alpha, x, incx, y, incy);
}
void qref_c_qgemv(char layout, char trans, int m, int n, double alpha, void* A, int lda, void* x,
                  int incx, double beta, void* y, int incy) {
  quadblas_qgemv(layout, trans, m, n, alpha, A, lda, x, incx, beta, y, incy);
}
void qref_c_qgemm(char layout, char transa, char transb, int m, int n, int k, double alpha,
                  void* A, int lda, void* B, int ldb, double beta, void* C, int ldc) {
  quadblas_qgemm(layout, transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}
void qref_set_num_threads(int t) { quadblas_set_num_threads(t); }

}  // extern "C"
