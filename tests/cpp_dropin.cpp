// A C++ program written against the reference's C++ interface
// (QuadBLAS::Vector / QuadBLAS::Matrix members, include/quadblas/quadblas.hpp
// and interface/cpp_classes.hpp of QuadBLAS 1.0.0), built unchanged against
// this library's header and libquadblas_gpu.so.
//
// Known answers first (the reference's tests/test_quadblas.cpp: dot of 1..10
// with ones is 55; 1e20 + 1 - 1e20 is 1; 2x2 gemm/gemv results), then the
// operations on the inputs read from argv[1], written to argv[2]:
//   input : int64 n, m, k; x[n], y[n], A[m*k] (row-major), B[k*m] (row-major),
//           v[k], w[m] (binary128, 16 bytes each)
//   output: dot(x, y); norm(x); x*2.5 + y (axpy); A.gemv(1.5, v, 0.5, w) row-major;
//           the same buffer as a column-major k x m matrix times the input w
//           (A^T w);
//           A.gemm(1, B, 0, C) row-major (m x m); the same buffers viewed
//           column-major (B^T A^T = (A B)^T stored column-major = A B row-major).
#include <stdio.h>
#include <stdlib.h>

#include <vector>

#include "quadblas/quadblas.hpp"

using QuadBLAS::Layout;

static int fail(const char* what) {
  fprintf(stderr, "FAIL: %s\n", what);
  return 1;
}

static bool same(Sleef_quad a, Sleef_quad b) { return memcmp(&a, &b, sizeof a) == 0; }

static int known_answers() {
  QuadBLAS::DefaultVector<> x(10), ones(10);
  for (int i = 0; i < 10; ++i) {
    x[i] = SLEEF_QUAD_C(i + 1);
    ones[i] = SLEEF_QUAD_C(1);
  }
  if (!same(x.dot(ones), SLEEF_QUAD_C(55))) return fail("dot(1..10, 1) == 55");
  QuadBLAS::DefaultVector<> a(3), b(3);
  a[0] = SLEEF_QUAD_C(1e20);
  a[1] = SLEEF_QUAD_C(1);
  a[2] = SLEEF_QUAD_C(-1e20);
  for (int i = 0; i < 3; ++i) b[i] = SLEEF_QUAD_C(1);
  if (!same(a.dot(b), SLEEF_QUAD_C(1))) return fail("1e20 + 1 - 1e20 == 1");
  QuadBLAS::MatrixRowMajor A(2, 2), B(2, 2), C(2, 2);
  A(0, 0) = SLEEF_QUAD_C(1); A(0, 1) = SLEEF_QUAD_C(2);
  A(1, 0) = SLEEF_QUAD_C(3); A(1, 1) = SLEEF_QUAD_C(4);
  B(0, 0) = SLEEF_QUAD_C(5); B(0, 1) = SLEEF_QUAD_C(6);
  B(1, 0) = SLEEF_QUAD_C(7); B(1, 1) = SLEEF_QUAD_C(8);
  A.gemm(SLEEF_QUAD_C(1), B, SLEEF_QUAD_C(0), C);
  if (!same(C(0, 0), SLEEF_QUAD_C(19)) || !same(C(0, 1), SLEEF_QUAD_C(22)) ||
      !same(C(1, 0), SLEEF_QUAD_C(43)) || !same(C(1, 1), SLEEF_QUAD_C(50)))
    return fail("2x2 gemm");
  QuadBLAS::VectorRowMajor v(2), w(2);
  v[0] = SLEEF_QUAD_C(1);
  v[1] = SLEEF_QUAD_C(1);
  A.gemv(SLEEF_QUAD_C(1), v, SLEEF_QUAD_C(0), w);
  if (!same(w[0], SLEEF_QUAD_C(3)) || !same(w[1], SLEEF_QUAD_C(7))) return fail("2x2 gemv");
  QuadBLAS::MatrixColMajor Ac(2, 2);
  Ac(0, 0) = SLEEF_QUAD_C(1); Ac(0, 1) = SLEEF_QUAD_C(2);
  Ac(1, 0) = SLEEF_QUAD_C(3); Ac(1, 1) = SLEEF_QUAD_C(4);
  QuadBLAS::VectorColMajor vc(2), wc(2);
  vc[0] = SLEEF_QUAD_C(1);
  vc[1] = SLEEF_QUAD_C(1);
  Ac.gemv(SLEEF_QUAD_C(1), vc, SLEEF_QUAD_C(0), wc);
  if (!same(wc[0], SLEEF_QUAD_C(3)) || !same(wc[1], SLEEF_QUAD_C(7))) return fail("2x2 col-major gemv");
  if (!same(x.norm() * x.norm(), SLEEF_QUAD_C(385)) && !(x.norm() > SLEEF_QUAD_C(19.62) &&
                                                         x.norm() < SLEEF_QUAD_C(19.63)))
    return fail("norm(1..10)");
  return 0;
}

int main(int argc, char** argv) {
  if (int rc = known_answers()) return rc;
  if (argc < 3) return 0;
  FILE* f = fopen(argv[1], "rb");
  if (!f) return fail("open input");
  int64_t hdr[3];
  if (fread(hdr, sizeof(int64_t), 3, f) != 3) return fail("read header");
  const size_t n = (size_t)hdr[0], m = (size_t)hdr[1], k = (size_t)hdr[2];
  QuadBLAS::DefaultVector<> x(n), y(n), v(k), w(m), wt(m);
  QuadBLAS::MatrixRowMajor A(m, k), B(k, m), C(m, m);
  bool ok = fread(x.data(), 16, n, f) == n && fread(y.data(), 16, n, f) == n &&
            fread(A.data(), 16, m * k, f) == m * k && fread(B.data(), 16, k * m, f) == k * m &&
            fread(v.data(), 16, k, f) == k && fread(w.data(), 16, m, f) == m;
  fclose(f);
  if (!ok) return fail("read input");
  memcpy(static_cast<void*>(wt.data()), w.data(), 16 * m);

  std::vector<Sleef_quad> out;
  out.push_back(x.dot(y));
  out.push_back(x.norm());
  QuadBLAS::DefaultVector<> z(n);
  memcpy(static_cast<void*>(z.data()), y.data(), 16 * n);
  z.axpy(SLEEF_QUAD_C(2.5), x);
  out.insert(out.end(), z.data(), z.data() + n);
  A.gemv(SLEEF_QUAD_C(1.5), v, SLEEF_QUAD_C(0.5), w);
  out.insert(out.end(), w.data(), w.data() + m);
  // the row-major m x k buffer read as a column-major k x m matrix is A^T
  QuadBLAS::MatrixColMajor At(A.data(), k, m, k);
  QuadBLAS::VectorColMajor wv(wt.data(), m);  // w as read, before the gemv above
  QuadBLAS::VectorColMajor r(k);
  At.gemv(SLEEF_QUAD_C(1), wv, SLEEF_QUAD_C(0), r);
  out.insert(out.end(), r.data(), r.data() + k);
  A.gemm(SLEEF_QUAD_C(1), B, SLEEF_QUAD_C(0), C);
  out.insert(out.end(), C.data(), C.data() + m * m);
  // column-major: (B^T)(A^T) with B^T = B's buffer as m x k column-major
  QuadBLAS::MatrixColMajor Bt(B.data(), m, k, m), Atc(A.data(), k, m, k), Cc(m, m);
  Bt.gemm(SLEEF_QUAD_C(1), Atc, SLEEF_QUAD_C(0), Cc);
  out.insert(out.end(), Cc.data(), Cc.data() + m * m);

  FILE* g = fopen(argv[2], "wb");
  if (!g) return fail("open output");
  ok = fwrite(out.data(), 16, out.size(), g) == out.size();
  fclose(g);
  return ok ? 0 : fail("write output");
}
