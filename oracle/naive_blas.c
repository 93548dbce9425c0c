/*
 * Deterministic BLAS shim for the CPU oracle (test infrastructure only).
 *
 * The reference routes all block arithmetic through Fortran BLAS symbols
 * (blaslapack.h:19-27: dgemm_, daxpy_, ddot_, dnrm2_, sgemm_, saxpy_) and
 * links MKL (Makefile:5).  MKL is not pinned, so its last-ulp behaviour
 * cannot be reproduced.  This file *defines* those routines with a fixed
 * operation order so that the reference compiled against it, the C
 * restatement in bsm_oracle.c, and the GPU kernels all perform the same
 * sequence of IEEE-754 double operations:
 *
 *   gemm : for every C element, t = 0; t = fma(op(A)[i,l], op(B)[l,j], t)
 *          for l = 0..k-1 in order; then C = alpha*t (beta == 0) or
 *          C = alpha*t + beta*C (two products, one sum, no contraction).
 *   axpy : y[i] = fma(a, x[i], y[i])           (a = +-1 gives one add/sub)
 *   dot  : t = 0; t = fma(x[i], y[i], t) in order
 *   nrm2 : 32 "lanes"; lane l sums fma(x[i], x[i], s_l) over i = l, l+32, ...;
 *          then s_l += s_{l+o} for o = 16, 8, 4, 2, 1 (the warp-shuffle tree
 *          the GPU norm kernel uses); result sqrt(s_0).  No overflow
 *          scaling (the synthetic inputs stay far from the double range).
 *
 * Build with -ffp-contract=off so the compiler adds no fused operations.
 * LP64 Fortran ABI (int* sizes), as declared by the reference.
 */
#include <dlfcn.h>
#include <math.h>
#include <stddef.h>
#include <stdint.h>

#include "naive_blas.h"

/* Optional timing mode (CPU baseline only, never used for parity): forward
 * nb_dgemm to an ILP64 Fortran dgemm (numpy's bundled OpenBLAS exports it as
 * scipy_dgemm_64_), standing in for the MKL the reference links. */
typedef void (*ilp64_dgemm_t)(const char *, const char *, const int64_t *, const int64_t *, const int64_t *,
                              const double *, const double *, const int64_t *, const double *, const int64_t *,
                              const double *, double *, const int64_t *);
static ilp64_dgemm_t g_fwd_gemm = 0;

int nb_enable_fast_gemm(const char *lib_path) {
    if (!lib_path) {
        g_fwd_gemm = 0;
        return 0;
    }
    void *h = dlopen(lib_path, RTLD_NOW | RTLD_LOCAL);
    if (!h) return -1;
    g_fwd_gemm = (ilp64_dgemm_t)dlsym(h, "scipy_dgemm_64_");
    void (*set_threads)(int64_t) = (void (*)(int64_t))dlsym(h, "scipy_openblas_set_num_threads64_");
    if (set_threads) set_threads(1);
    return g_fwd_gemm ? 0 : -2;
}

static inline double opd(const double *M, int ld, int trans, int r, int c) {
    /* element (r, c) of op(M) for a column-major M with leading dimension ld */
    return trans ? M[(size_t)c + (size_t)r * (size_t)ld] : M[(size_t)r + (size_t)c * (size_t)ld];
}

static inline int is_trans(const char *t) { return *t == 't' || *t == 'T' || *t == 'c' || *t == 'C'; }

void nb_dgemm(int ta, int tb, int m, int n, int k, double alpha, const double *A, int lda,
              const double *B, int ldb, double beta, double *C, int ldc) {
    if (g_fwd_gemm) {
        if (m <= 0 || n <= 0) return;
        const char cta = ta ? 'T' : 'N', ctb = tb ? 'T' : 'N';
        const int64_t M = m, N = n, K = k, LDA = lda, LDB = ldb, LDC = ldc;
        g_fwd_gemm(&cta, &ctb, &M, &N, &K, &alpha, A, &LDA, B, &LDB, &beta, C, &LDC);
        return;
    }
    for (int j = 0; j < n; ++j) {
        for (int i = 0; i < m; ++i) {
            double t = 0.0;
            for (int l = 0; l < k; ++l) t = fma(opd(A, lda, ta, i, l), opd(B, ldb, tb, l, j), t);
            double *c = &C[(size_t)i + (size_t)j * (size_t)ldc];
            if (beta == 0.0) {
                *c = alpha * t;
            } else {
                double p = alpha * t;
                double q = beta * (*c);
                *c = p + q;
            }
        }
    }
}

double nb_nrm2(int n, const double *x, int incx) {
    double s[32];
    for (int l = 0; l < 32; ++l) {
        double acc = 0.0;
        for (int i = l; i < n; i += 32) {
            double v = x[(size_t)i * (size_t)incx];
            acc = fma(v, v, acc);
        }
        s[l] = acc;
    }
    for (int o = 16; o >= 1; o >>= 1)
        for (int l = 0; l < o; ++l) s[l] = s[l] + s[l + o];
    return sqrt(s[0]);
}

void nb_daxpy(int n, double a, const double *x, int incx, double *y, int incy) {
    for (int i = 0; i < n; ++i) {
        double *yy = &y[(size_t)i * (size_t)incy];
        *yy = fma(a, x[(size_t)i * (size_t)incx], *yy);
    }
}

double nb_ddot(int n, const double *x, int incx, const double *y, int incy) {
    double t = 0.0;
    for (int i = 0; i < n; ++i) t = fma(x[(size_t)i * (size_t)incx], y[(size_t)i * (size_t)incy], t);
    return t;
}

/* ---- Fortran-ABI entry points the reference links against ---- */

void dgemm_(const char *ta, const char *tb, const int *m, const int *n, const int *k, const double *alpha,
            const double *A, const int *lda, const double *B, const int *ldb, const double *beta, double *C,
            const int *ldc) {
    nb_dgemm(is_trans(ta), is_trans(tb), *m, *n, *k, *alpha, A, *lda, B, *ldb, *beta, C, *ldc);
}

void daxpy_(const int *n, const double *a, const double *x, const int *incx, double *y, const int *incy) {
    nb_daxpy(*n, *a, x, *incx, y, *incy);
}

double ddot_(const int *n, const double *x, const int *incx, const double *y, const int *incy) {
    return nb_ddot(*n, x, *incx, y, *incy);
}

double dnrm2_(const int *n, const double *x, const int *incx) { return nb_nrm2(*n, x, *incx); }

void sgemm_(const char *ta, const char *tb, const int *m, const int *n, const int *k, const float *alpha,
            const float *A, const int *lda, const float *B, const int *ldb, const float *beta, float *C,
            const int *ldc) {
    int TA = is_trans(ta), TB = is_trans(tb);
    for (int j = 0; j < *n; ++j)
        for (int i = 0; i < *m; ++i) {
            float t = 0.0f;
            for (int l = 0; l < *k; ++l) {
                float a = TA ? A[l + (size_t)i * *lda] : A[i + (size_t)l * *lda];
                float b = TB ? B[j + (size_t)l * *ldb] : B[l + (size_t)j * *ldb];
                t = fmaf(a, b, t);
            }
            float *c = &C[i + (size_t)j * *ldc];
            *c = (*beta == 0.0f) ? (*alpha) * t : (*alpha) * t + (*beta) * (*c);
        }
}

void saxpy_(const int *n, const float *a, const float *x, const int *incx, float *y, const int *incy) {
    for (int i = 0; i < *n; ++i) y[(size_t)i * *incy] = fmaf(*a, x[(size_t)i * *incx], y[(size_t)i * *incy]);
}
