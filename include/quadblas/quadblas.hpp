// quadblas.hpp — C++ front end of libquadblas_gpu.so with the names of the
// reference's header-only library (include/quadblas/quadblas.hpp of
// QuadBLAS 1.0.0): QuadBLAS::Layout, dot/axpy/gemv/gemm, Vector<L>,
// Matrix<L>, aligned_alloc/aligned_free, get/set_num_threads.  The
// arithmetic runs on the GPU through the C ABI in ../quadblas_gpu.h.
//
// Sleef_quad: when SLEEF's <sleefquad.h> is included first (it defines
// SLEEF_QUAD_C) its type is used; otherwise the host compiler's IEEE
// binary128 type (long double on AArch64, __float128 elsewhere where GCC or
// Clang provide it).
//
// Errors: the reference has no error reporting; these functions throw
// QuadBLAS::Error (a std::runtime_error) when the GPU call fails.
#ifndef QBLAS_GB300_QUADBLAS_HPP
#define QBLAS_GB300_QUADBLAS_HPP

#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cstddef>
#include <stdexcept>
#include <string>

#include "../quadblas_gpu.h"

#if !defined(SLEEF_QUAD_C)
#if defined(__aarch64__)
typedef long double Sleef_quad;
#elif defined(__SIZEOF_FLOAT128__)
typedef __float128 Sleef_quad;
#else
#error "quadblas.hpp needs a 16-byte IEEE binary128 type (include <sleefquad.h> first)"
#endif
#define SLEEF_QUAD_C(x) ((Sleef_quad)(x))
#endif

static_assert(sizeof(Sleef_quad) == 16, "Sleef_quad must be IEEE binary128");

namespace QuadBLAS {

// core/types.hpp:8
enum class Layout { RowMajor, ColMajor };

// core/constants.hpp:18
constexpr size_t ALIGNMENT = 32;
constexpr const char* VERSION = "1.0.0";
constexpr int VERSION_MAJOR = 1;
constexpr int VERSION_MINOR = 0;
constexpr int VERSION_PATCH = 0;

class Error : public std::runtime_error {
 public:
  explicit Error(int code)
      : std::runtime_error(std::string("quadblas_gpu: ") + quadblas_error_string(code)),
        code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

inline void check(int status) {
  if (status != QBLAS_OK) throw Error(status);
}

// memory/allocation.hpp:19-41
template <typename T>
inline T* aligned_alloc(size_t count) {
  void* p = nullptr;
  if (posix_memalign(&p, ALIGNMENT, count * sizeof(T)) != 0) p = nullptr;
  return static_cast<T*>(p);
}
template <typename T>
inline void aligned_free(T* p) {
  free(p);
}

// threading/openmp_utils.hpp:10-24 (recorded only; no host thread pool)
inline int get_num_threads() { return quadblas_get_num_threads(); }
inline void set_num_threads(int n) { quadblas_set_num_threads(n); }

inline char layout_char(Layout l) { return l == Layout::ColMajor ? 'C' : 'R'; }

// algorithms/level1.hpp:80
inline Sleef_quad dot(size_t n, const Sleef_quad* x, size_t incx, const Sleef_quad* y,
                      size_t incy) {
  Sleef_quad r;
  check(quadblas_qdot_q((int64_t)n, x, (int64_t)incx, y, (int64_t)incy, &r));
  return r;
}

// algorithms/level1.hpp:190
inline void axpy(size_t n, Sleef_quad alpha, const Sleef_quad* x, size_t incx, Sleef_quad* y,
                 size_t incy) {
  check(quadblas_qaxpy_q((int64_t)n, &alpha, x, (int64_t)incx, y, (int64_t)incy));
}

// algorithms/level2.hpp:85
inline void gemv(Layout layout, size_t m, size_t n, Sleef_quad alpha, const Sleef_quad* A,
                 size_t lda, const Sleef_quad* x, size_t incx, Sleef_quad beta, Sleef_quad* y,
                 size_t incy) {
  check(quadblas_qgemv_q(layout_char(layout), 'N', (int64_t)m, (int64_t)n, &alpha, A,
                         (int64_t)lda, x, (int64_t)incx, &beta, y, (int64_t)incy));
}

// algorithms/level3.hpp:215
inline void gemm(Layout layout, size_t m, size_t n, size_t k, Sleef_quad alpha,
                 const Sleef_quad* A, size_t lda, const Sleef_quad* B, size_t ldb,
                 Sleef_quad beta, Sleef_quad* C, size_t ldc) {
  check(quadblas_qgemm_q(layout_char(layout), 'N', 'N', (int64_t)m, (int64_t)n, (int64_t)k,
                         &alpha, A, (int64_t)lda, B, (int64_t)ldb, &beta, C, (int64_t)ldc));
}

inline Sleef_quad nrm2(size_t n, const Sleef_quad* x, size_t incx) {
  Sleef_quad r;
  check(quadblas_qnrm2_q((int64_t)n, x, (int64_t)incx, &r));
  return r;
}

template <Layout layout>
class Matrix;

// interface/cpp_classes.hpp:18-82
template <Layout layout>
class Vector {
 public:
  explicit Vector(size_t size) : size_(size), stride_(1), owns_(true) {
    data_ = aligned_alloc<Sleef_quad>(size ? size : 1);
    if (!data_) throw std::bad_alloc();
    memset(static_cast<void*>(data_), 0, sizeof(Sleef_quad) * size);
  }
  Vector(Sleef_quad* data, size_t size, size_t stride = 1)
      : data_(data), size_(size), stride_(stride), owns_(false) {}
  ~Vector() {
    if (owns_) aligned_free(data_);
  }
  Vector(Vector&& o) noexcept : data_(o.data_), size_(o.size_), stride_(o.stride_), owns_(o.owns_) {
    o.owns_ = false;
  }
  Vector(const Vector&) = delete;
  Vector& operator=(const Vector&) = delete;

  Sleef_quad& operator[](size_t i) { return data_[i * stride_]; }
  const Sleef_quad& operator[](size_t i) const { return data_[i * stride_]; }
  size_t size() const { return size_; }
  size_t stride() const { return stride_; }
  Sleef_quad* data() { return data_; }
  const Sleef_quad* data() const { return data_; }

  Sleef_quad dot(const Vector& other) const {
    return QuadBLAS::dot(size_, data_, stride_, other.data_, other.stride_);
  }
  void axpy(Sleef_quad alpha, const Vector& other) {
    QuadBLAS::axpy(size_, alpha, other.data_, other.stride_, data_, stride_);
  }
  Sleef_quad norm() const { return QuadBLAS::nrm2(size_, data_, stride_); }

 private:
  Sleef_quad* data_;
  size_t size_, stride_;
  bool owns_;
};

// interface/cpp_classes.hpp:84-155
template <Layout layout>
class Matrix {
 public:
  Matrix(size_t rows, size_t cols) : rows_(rows), cols_(cols), ld_(cols), owns_(true) {
    data_ = aligned_alloc<Sleef_quad>(rows * cols != 0 ? rows * cols : 1);
    if (!data_) throw std::bad_alloc();
    memset(static_cast<void*>(data_), 0, sizeof(Sleef_quad) * rows * cols);
  }
  Matrix(Sleef_quad* data, size_t rows, size_t cols, size_t ld = 0)
      : data_(data), rows_(rows), cols_(cols), ld_(ld == 0 ? cols : ld), owns_(false) {}
  ~Matrix() {
    if (owns_) aligned_free(data_);
  }
  Matrix(Matrix&& o) noexcept
      : data_(o.data_), rows_(o.rows_), cols_(o.cols_), ld_(o.ld_), owns_(o.owns_) {
    o.owns_ = false;
  }
  Matrix(const Matrix&) = delete;
  Matrix& operator=(const Matrix&) = delete;

  Sleef_quad& operator()(size_t i, size_t j) {
    return layout == Layout::RowMajor ? data_[i * ld_ + j] : data_[j * ld_ + i];
  }
  const Sleef_quad& operator()(size_t i, size_t j) const {
    return layout == Layout::RowMajor ? data_[i * ld_ + j] : data_[j * ld_ + i];
  }
  size_t rows() const { return rows_; }
  size_t cols() const { return cols_; }
  size_t leading_dimension() const { return ld_; }
  Sleef_quad* data() { return data_; }
  const Sleef_quad* data() const { return data_; }

  void gemv(Sleef_quad alpha, const Vector<layout>& x, Sleef_quad beta, Vector<layout>& y) const {
    QuadBLAS::gemv(layout, rows_, cols_, alpha, data_, ld_, x.data(), x.stride(), beta, y.data(),
                   y.stride());
  }
  void gemm(Sleef_quad alpha, const Matrix& B, Sleef_quad beta, Matrix& C) const {
    QuadBLAS::gemm(layout, rows_, B.cols(), cols_, alpha, data_, ld_, B.data(),
                   B.leading_dimension(), beta, C.data(), C.leading_dimension());
  }

 private:
  Sleef_quad* data_;
  size_t rows_, cols_, ld_;
  bool owns_;
};

using VectorRowMajor = Vector<Layout::RowMajor>;
using VectorColMajor = Vector<Layout::ColMajor>;
using MatrixRowMajor = Matrix<Layout::RowMajor>;
using MatrixColMajor = Matrix<Layout::ColMajor>;
template <Layout layout = Layout::RowMajor>
using DefaultVector = Vector<layout>;
template <Layout layout = Layout::RowMajor>
using DefaultMatrix = Matrix<layout>;

}  // namespace QuadBLAS

#endif  // QBLAS_GB300_QUADBLAS_HPP
