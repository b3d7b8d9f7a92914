/* Test infrastructure: NOT part of the product.
 *
 * Fortran BLAS entry points for the reference build with BLAS enabled
 * (ref_harness_blas, oracle/ref_build.mk): the image has no system BLAS, but
 * SciPy ships OpenBLAS with every Fortran symbol renamed with a "scipy_"
 * prefix.  Each function here forwards one name Armadillo calls to that
 * library, with the Fortran calling convention (every argument by address;
 * the hidden character-length arguments gfortran-style callers append are
 * passed through).  Threads: set OPENBLAS_NUM_THREADS=1, as the reference's
 * own OpenMP loops call BLAS from every thread. */
#include <stddef.h>

typedef int blas_int;

void scipy_dgemm_(const char*, const char*, const blas_int*, const blas_int*, const blas_int*, const double*,
                  const double*, const blas_int*, const double*, const blas_int*, const double*, double*,
                  const blas_int*, size_t, size_t);
void scipy_dgemv_(const char*, const blas_int*, const blas_int*, const double*, const double*, const blas_int*,
                  const double*, const blas_int*, const double*, double*, const blas_int*, size_t);
void scipy_dsyrk_(const char*, const char*, const blas_int*, const blas_int*, const double*, const double*,
                  const blas_int*, const double*, double*, const blas_int*, size_t, size_t);
double scipy_ddot_(const blas_int*, const double*, const blas_int*, const double*, const blas_int*);
double scipy_dnrm2_(const blas_int*, const double*, const blas_int*);
double scipy_dasum_(const blas_int*, const double*, const blas_int*);

void dgemm_(const char* ta, const char* tb, const blas_int* m, const blas_int* n, const blas_int* k,
            const double* alpha, const double* A, const blas_int* lda, const double* B, const blas_int* ldb,
            const double* beta, double* C, const blas_int* ldc, size_t la, size_t lb)
{
  scipy_dgemm_(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, la, lb);
}

void dgemv_(const char* t, const blas_int* m, const blas_int* n, const double* alpha, const double* A,
            const blas_int* lda, const double* x, const blas_int* incx, const double* beta, double* y,
            const blas_int* incy, size_t lt)
{
  scipy_dgemv_(t, m, n, alpha, A, lda, x, incx, beta, y, incy, lt);
}

void dsyrk_(const char* uplo, const char* t, const blas_int* n, const blas_int* k, const double* alpha,
            const double* A, const blas_int* lda, const double* beta, double* C, const blas_int* ldc, size_t lu,
            size_t lt)
{
  scipy_dsyrk_(uplo, t, n, k, alpha, A, lda, beta, C, ldc, lu, lt);
}

double ddot_(const blas_int* n, const double* x, const blas_int* incx, const double* y, const blas_int* incy)
{
  return scipy_ddot_(n, x, incx, y, incy);
}

double dnrm2_(const blas_int* n, const double* x, const blas_int* incx) { return scipy_dnrm2_(n, x, incx); }

double dasum_(const blas_int* n, const double* x, const blas_int* incx) { return scipy_dasum_(n, x, incx); }
