/* Deterministic BLAS shim shared by the C oracle and the compiled reference
 * (test infrastructure only; see naive_blas.c for the operation order). */
#ifndef BSG_ORACLE_NAIVE_BLAS_H
#define BSG_ORACLE_NAIVE_BLAS_H
#ifdef __cplusplus
extern "C" {
#endif

void nb_dgemm(int ta, int tb, int m, int n, int k, double alpha, const double *A, int lda,
              const double *B, int ldb, double beta, double *C, int ldc);
double nb_nrm2(int n, const double *x, int incx);
void nb_daxpy(int n, double a, const double *x, int incx, double *y, int incy);
double nb_ddot(int n, const double *x, int incx, const double *y, int incy);
/* timing mode only: route nb_dgemm to an ILP64 OpenBLAS (NULL restores the
 * deterministic loop); returns 0 on success */
int nb_enable_fast_gemm(const char *lib_path);

#ifdef __cplusplus
}
#endif
#endif
