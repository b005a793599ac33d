/*
 * ORACLE / TEST INFRASTRUCTURE ONLY. The legacy cuBLAS calls of the
 * reference's GPU sources, on host memory, through Fortran BLAS (the OpenBLAS
 * that scipy bundles; see blas_trampoline.c). Same argument meaning as the
 * legacy cuBLAS API (column-major, leading dimensions).
 */
#ifndef CESA_EMU_CUBLAS_H_
#define CESA_EMU_CUBLAS_H_

typedef int cublasStatus;

cublasStatus cublasInit();
cublasStatus cublasShutdown();
void cublasSgemv(char trans, int m, int n, float alpha, const float* A, int lda, const float* x, int incx,
                 float beta, float* y, int incy);
void cublasSaxpy(int n, float alpha, const float* x, int incx, float* y, int incy);
float cublasSasum(int n, const float* x, int incx);
void cublasSscal(int n, float alpha, float* x, int incx);
void cublasSgemm(char transa, char transb, int m, int n, int k, float alpha, const float* A, int lda,
                 const float* B, int ldb, float beta, float* C, int ldc);

#endif
