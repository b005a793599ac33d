/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * The reference calls Fortran BLAS/LAPACK (sgemm_, sgemv_, saxpy_, sasum_,
 * sscal_, dsyev_; src/emicp_cpu.cpp:33-43, src/findRTfromS.cpp:101-106).
 * No system BLAS exists here, so these forward to the OpenBLAS build that
 * scipy bundles (symbols carry a "scipy_" prefix). The hidden Fortran
 * string-length arguments are passed explicitly as 1.
 */
#include <stddef.h>

extern int scipy_sgemm_(const char*, const char*, const int*, const int*, const int*, const float*,
                        const float*, const int*, const float*, const int*, const float*, float*,
                        const int*, size_t, size_t);
extern int scipy_sgemv_(const char*, const int*, const int*, const float*, const float*, const int*,
                        const float*, const int*, const float*, float*, const int*, size_t);
extern int scipy_saxpy_(const int*, const float*, const float*, const int*, float*, const int*);
extern float scipy_sasum_(const int*, const float*, const int*);
extern int scipy_sscal_(const int*, const float*, float*, const int*);
extern int scipy_dsyev_(const char*, const char*, const int*, double*, const int*, double*, double*,
                        const int*, int*, size_t, size_t);

int sgemm_(const char* ta, const char* tb, const int* m, const int* n, const int* k, const float* al,
           const float* a, const int* lda, const float* b, const int* ldb, const float* be, float* c,
           const int* ldc) {
  return scipy_sgemm_(ta, tb, m, n, k, al, a, lda, b, ldb, be, c, ldc, 1, 1);
}
int sgemv_(const char* tr, const int* m, const int* n, const float* al, const float* a,
           const int* lda, const float* x, const int* incx, const float* be, float* y,
           const int* incy) {
  return scipy_sgemv_(tr, m, n, al, a, lda, x, incx, be, y, incy, 1);
}
int saxpy_(const int* n, const float* sa, const float* sx, const int* incx, float* sy,
           const int* incy) {
  return scipy_saxpy_(n, sa, sx, incx, sy, incy);
}
float sasum_(const int* n, const float* sx, const int* incx) { return scipy_sasum_(n, sx, incx); }
int sscal_(const int* n, const float* sa, float* sx, const int* incx) {
  return scipy_sscal_(n, sa, sx, incx);
}
int dsyev_(char* jobz, char* uplo, int* n, double* a, int* lda, double* w, double* work, int* lwork,
           int* info) {
  return scipy_dsyev_(jobz, uplo, n, a, lda, w, work, lwork, info, 1, 1);
}
