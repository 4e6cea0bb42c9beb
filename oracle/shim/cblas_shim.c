/* Plain-loop CBLAS subset for building the reference evaluator here
 * (see external/cblas-prototypes/cblas.h).  Semantics follow the CBLAS standard:
 * C = alpha op(A) op(B) + beta C and y = alpha op(A) x + beta y, row- or
 * column-major.  Test infrastructure only; never linked into the GPU engine. */
#include "external/cblas-prototypes/cblas.h"

static double at(CBLAS_LAYOUT layout, const double* a, int lda, int i, int j) {
  return layout == CblasRowMajor ? a[(long)i * lda + j] : a[(long)j * lda + i];
}

void cblas_dgemm(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE transa, CBLAS_TRANSPOSE transb, int m, int n,
                 int k, double alpha, const double* a, int lda, const double* b, int ldb, double beta,
                 double* c, int ldc) {
  for (int i = 0; i < m; ++i) {
    for (int j = 0; j < n; ++j) {
      double s = 0.0;
      for (int p = 0; p < k; ++p) {
        const double av = transa == CblasNoTrans ? at(layout, a, lda, i, p) : at(layout, a, lda, p, i);
        const double bv = transb == CblasNoTrans ? at(layout, b, ldb, p, j) : at(layout, b, ldb, j, p);
        s += av * bv;
      }
      double* cij = layout == CblasRowMajor ? &c[(long)i * ldc + j] : &c[(long)j * ldc + i];
      *cij = (beta == 0.0 ? 0.0 : beta * *cij) + alpha * s;
    }
  }
}

void cblas_dgemv(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE trans, int m, int n, double alpha,
                 const double* a, int lda, const double* x, int incx, double beta, double* y,
                 int incy) {
  const int rows = trans == CblasNoTrans ? m : n;
  const int cols = trans == CblasNoTrans ? n : m;
  for (int i = 0; i < rows; ++i) {
    double s = 0.0;
    for (int j = 0; j < cols; ++j) {
      const double av = trans == CblasNoTrans ? at(layout, a, lda, i, j) : at(layout, a, lda, j, i);
      s += av * x[(long)j * incx];
    }
    double* yi = &y[(long)i * incy];
    *yi = (beta == 0.0 ? 0.0 : beta * *yi) + alpha * s;
  }
}

void cblas_dcopy(int n, const double* x, int incx, double* y, int incy) {
  for (int i = 0; i < n; ++i) y[(long)i * incy] = x[(long)i * incx];
}

double cblas_ddot(int n, const double* x, int incx, const double* y, int incy) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += x[(long)i * incx] * y[(long)i * incy];
  return s;
}
