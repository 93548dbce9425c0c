/*
 * CPU oracle: a plain-C restatement of the reference's block-sparse matrix,
 * screened block GEMM, hybrid Strassen-Winograd/sparse recursion and the
 * occupied RI-K step.  TEST INFRASTRUCTURE ONLY: tests/, the smoke check and
 * bench.py's CPU-baseline leg may call it, nothing in the product does.
 * Every function names the reference file:line it restates.
 */
#ifndef BSG_ORACLE_H
#define BSG_ORACLE_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct ob_bsm {
    size_t nr, nc, bsr, bsc, nrb, ncb;
    double thresh;
    double **blk; /* nrb*ncb block pointers, block (r,c) at r + c*nrb; NULL = absent */
    int *brows;   /* rows of each present block (0 when absent) */
    int *bcols;   /* cols of each present block (0 when absent) */
    double *norm; /* cached Frobenius norm of each block (0 when absent) */
} ob_bsm;

/* status codes: 0 ok, otherwise a precondition the reference would assert on */
enum { OB_OK = 0, OB_EDIM = 1, OB_EPRECOND = 2, OB_ENOMEM = 3 };

ob_bsm *ob_create(size_t nr, size_t nc, size_t bsr, size_t bsc, double thresh);
void ob_free(ob_bsm *m);
int ob_copy(ob_bsm *dst, const ob_bsm *src);
int ob_copy_from_dense(ob_bsm *m, const double *in);
void ob_fill(ob_bsm *m, double val);
void ob_zero(ob_bsm *m);
void ob_scale(ob_bsm *m, double s);
int ob_add(ob_bsm *m, const ob_bsm *rhs);
int ob_sub(ob_bsm *m, const ob_bsm *rhs);
int ob_add_transpose(ob_bsm *m, const ob_bsm *rhs);
void ob_calc_norms(ob_bsm *m);
void ob_recompress(ob_bsm *m);
double ob_frobenius_norm(const ob_bsm *m);
size_t ob_no_of_alloc_blocks(const ob_bsm *m);
void ob_to_dense(const ob_bsm *m, double *out);
void ob_get_mask(const ob_bsm *m, uint8_t *mask);
void ob_get_norms(const ob_bsm *m, double *norms);
double ob_dot(const ob_bsm *a, const ob_bsm *b, double thresh);
int ob_matmult(ob_bsm *C, const ob_bsm *A, int tA, const ob_bsm *B, int tB, double thresh, double alpha,
               double beta, uint64_t *nsig_out);

/* Strassen dry run: tree bits for levels 0..L-1 concatenated (level l holds
 * ceil(nb/2^(l+1))^3 entries, index i + j*n + k*n*n), flops per level 0..L. */
int ob_strassen_dryrun(const ob_bsm *A, const ob_bsm *B, double thresh_per_block, int *n_levels,
                       uint8_t *tree_out, size_t tree_cap, uint64_t *flops_per_level);
int ob_matmult_strassen_sparse(ob_bsm *C, const ob_bsm *A, const ob_bsm *B, double thresh,
                               size_t min_size_for_strassen);

/* occ-RI-K step (occ_ri_k_step.cpp:83-130) with n_part OpenMP-static
 * partitions of P whose partial K's are summed in partition order. */
int ob_rik_occ_step(size_t n_bf, size_t n_aux, size_t n_occ, size_t n_vec2, const double *ints,
                    const uint64_t *keys, const double *c_occ, size_t bs, double thresh, int n_part,
                    double *k_out);
/* symmetric K_mn = sum_{P,i} mui_P(m,i) mui_P(n,i) on the occ step's mui_P
 * (occ_ri_k_step.cpp:102-108), per P matmult(Ks, mui, N, mui, T, thresh, 1, 1),
 * partitions as above; kmn_out n_bf x n_bf column-major */
int ob_rik_kmn_step(size_t n_bf, size_t n_aux, size_t n_occ, size_t n_vec2, const double *ints,
                    const uint64_t *keys, const double *c_occ, size_t bs, double thresh, int n_part,
                    double *kmn_out);
/* dense occ-RI-K (occ_ri_k_step.cpp:39-77) on the same partition rule */
int ob_rik_occ_dense(size_t n_bf, size_t n_aux, size_t n_occ, size_t n_vec2, const double *ints,
                     const uint64_t *keys, const double *c_occ, int n_part, double *k_out);
/* 3c->2c transform (3c_2c_transform.cpp:44-57) */
int ob_3c2c_transform(size_t n_vec2, size_t n_aux, const double *ints_3c, const double *v_m12, size_t bs,
                      double thresh, double *out);

#ifdef __cplusplus
}
#endif
#endif
