/*
 * CPU oracle (TEST INFRASTRUCTURE ONLY): plain-C restatement of the reference's
 * BlockSparseMatrix (blocksparsematrix.hpp), screened block GEMM, hybrid
 * Strassen-Winograd / sparse recursion (strassen.hpp) and the occ-RI-K and
 * 3c->2c drivers.  Arithmetic goes through the deterministic shim in
 * naive_blas.c, which is also what the compiled reference links against, so
 * the two agree bit for bit.  Build with -ffp-contract=off.
 */
#include "bsm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "naive_blas.h"

static size_t ceil_div(size_t a, size_t b) { return a == 0 ? 0 : 1 + (a - 1) / b; } /* utils.hpp:6-12 */

static size_t nat_rows(const ob_bsm *m, size_t rb) {
    size_t e = (rb + 1) * m->bsr;
    if (e > m->nr) e = m->nr;
    return e - rb * m->bsr;
}
static size_t nat_cols(const ob_bsm *m, size_t cb) {
    size_t e = (cb + 1) * m->bsc;
    if (e > m->nc) e = m->nc;
    return e - cb * m->bsc;
}

static void drop_block(ob_bsm *m, size_t b) {
    free(m->blk[b]);
    m->blk[b] = NULL;
    m->brows[b] = m->bcols[b] = 0;
    m->norm[b] = 0.0; /* a default-constructed Mat has norm 0 (matrix.h:71) */
}

static double *alloc_block(ob_bsm *m, size_t b, int rows, int cols) {
    free(m->blk[b]);
    m->blk[b] = (double *)malloc(sizeof(double) * (size_t)(rows > 0 ? rows : 1) * (size_t)(cols > 0 ? cols : 1));
    m->brows[b] = rows;
    m->bcols[b] = cols;
    return m->blk[b];
}

/* BlockSparseMatrix(nr,nc,bsr,bsc,thresh) blocksparsematrix.hpp:5-15 */
ob_bsm *ob_create(size_t nr, size_t nc, size_t bsr, size_t bsc, double thresh) {
    ob_bsm *m = (ob_bsm *)calloc(1, sizeof(ob_bsm));
    m->nr = nr;
    m->nc = nc;
    m->bsr = bsr;
    m->bsc = bsc;
    m->nrb = ceil_div(nr, bsr);
    m->ncb = ceil_div(nc, bsc);
    m->thresh = thresh;
    size_t nb = m->nrb * m->ncb;
    m->blk = (double **)calloc(nb ? nb : 1, sizeof(double *));
    m->brows = (int *)calloc(nb ? nb : 1, sizeof(int));
    m->bcols = (int *)calloc(nb ? nb : 1, sizeof(int));
    m->norm = (double *)calloc(nb ? nb : 1, sizeof(double));
    return m;
}

void ob_free(ob_bsm *m) {
    if (!m) return;
    for (size_t b = 0; b < m->nrb * m->ncb; ++b) free(m->blk[b]);
    free(m->blk);
    free(m->brows);
    free(m->bcols);
    free(m->norm);
    free(m);
}

/* copy assignment (occ_ri_k_step.cpp:112 `ijs = ij`): blocks and cached norms */
int ob_copy(ob_bsm *dst, const ob_bsm *src) {
    if (dst->nrb * dst->ncb != src->nrb * src->ncb) return OB_EDIM;
    dst->nr = src->nr;
    dst->nc = src->nc;
    dst->bsr = src->bsr;
    dst->bsc = src->bsc;
    dst->nrb = src->nrb;
    dst->ncb = src->ncb;
    dst->thresh = src->thresh;
    for (size_t b = 0; b < src->nrb * src->ncb; ++b) {
        if (src->blk[b]) {
            double *d = alloc_block(dst, b, src->brows[b], src->bcols[b]);
            memcpy(d, src->blk[b], sizeof(double) * (size_t)src->brows[b] * (size_t)src->bcols[b]);
        } else {
            drop_block(dst, b);
        }
        dst->norm[b] = src->norm[b];
    }
    return OB_OK;
}

/* copy_from_input_array blocksparsematrix.hpp:35-61: copy, norm, drop if
 * norm < thresh*bsr*bsc */
int ob_copy_from_dense(ob_bsm *m, const double *in) {
    const double tpb = m->thresh * (double)(m->bsc * m->bsr);
    for (size_t rcb = 0; rcb < m->nrb * m->ncb; ++rcb) {
        size_t cb = rcb / m->nrb, rb = rcb % m->nrb;
        int rs = (int)nat_rows(m, rb), cs = (int)nat_cols(m, cb);
        double *d = alloc_block(m, rcb, rs, cs);
        for (int c = 0; c < cs; ++c)
            memcpy(&d[(size_t)c * rs], &in[rb * m->bsr + (cb * m->bsc + (size_t)c) * m->nr], sizeof(double) * rs);
        double est = nb_nrm2(rs * cs, d, 1);
        m->norm[rcb] = est;
        if (est < tpb) drop_block(m, rcb);
    }
    return OB_OK;
}

/* fill_with_values blocksparsematrix.hpp:84-101 with Matrix(val,...) norm
 * sqrt(n)*val matrix.hpp:27-33 */
void ob_fill(ob_bsm *m, double val) {
    for (size_t rcb = 0; rcb < m->nrb * m->ncb; ++rcb) {
        size_t cb = rcb / m->nrb, rb = rcb % m->nrb;
        int rs = (int)nat_rows(m, rb), cs = (int)nat_cols(m, cb);
        double *d = alloc_block(m, rcb, rs, cs);
        for (int i = 0; i < rs * cs; ++i) d[i] = val;
        m->norm[rcb] = sqrt((double)((size_t)rs * (size_t)cs)) * val;
    }
}

/* zero() blocksparsematrix.hpp:79-82 */
void ob_zero(ob_bsm *m) {
    for (size_t b = 0; b < m->nrb * m->ncb; ++b) drop_block(m, b);
}

/* scale() blocksparsematrix.hpp:71-77; the cached norm is multiplied by
 * scale^2 (reference quirk, kept) */
void ob_scale(ob_bsm *m, double s) {
    for (size_t b = 0; b < m->nrb * m->ncb; ++b) {
        if (m->blk[b])
            for (int i = 0; i < m->brows[b] * m->bcols[b]; ++i) m->blk[b][i] = m->blk[b][i] * s;
    }
    for (size_t b = 0; b < m->nrb * m->ncb; ++b) m->norm[b] = m->norm[b] * (s * s);
}

static int same_shape(const ob_bsm *a, const ob_bsm *b) {
    return a->nrb == b->nrb && a->ncb == b->ncb && a->nr == b->nr && a->nc == b->nc;
}

/* operator+= blocksparsematrix.hpp:170-194 (norms are not refreshed, :190) */
int ob_add(ob_bsm *m, const ob_bsm *rhs) {
    if (!same_shape(m, rhs)) return OB_EDIM;
    for (size_t b = 0; b < m->nrb * m->ncb; ++b) {
        if (!rhs->blk[b]) continue;
        int n = rhs->brows[b] * rhs->bcols[b];
        if (!m->blk[b]) {
            double *d = alloc_block(m, b, rhs->brows[b], rhs->bcols[b]);
            memcpy(d, rhs->blk[b], sizeof(double) * (size_t)n);
            m->norm[b] = rhs->norm[b];
        } else {
            if (m->brows[b] != rhs->brows[b] || m->bcols[b] != rhs->bcols[b]) return OB_EDIM;
            nb_daxpy(n, 1.0, rhs->blk[b], 1, m->blk[b], 1);
        }
    }
    return OB_OK;
}

/* operator-= blocksparsematrix.hpp:196-221: an absent lhs block becomes a
 * plain copy of rhs (reference quirk, kept); norms are refreshed */
int ob_sub(ob_bsm *m, const ob_bsm *rhs) {
    if (!same_shape(m, rhs)) return OB_EDIM;
    for (size_t b = 0; b < m->nrb * m->ncb; ++b) {
        if (!rhs->blk[b]) continue;
        int n = rhs->brows[b] * rhs->bcols[b];
        if (!m->blk[b]) {
            double *d = alloc_block(m, b, rhs->brows[b], rhs->bcols[b]);
            memcpy(d, rhs->blk[b], sizeof(double) * (size_t)n);
        } else {
            if (m->brows[b] != rhs->brows[b] || m->bcols[b] != rhs->bcols[b]) return OB_EDIM;
            nb_daxpy(n, -1.0, rhs->blk[b], 1, m->blk[b], 1);
        }
        m->norm[b] = nb_nrm2(n, m->blk[b], 1);
    }
    return OB_OK;
}

/* add_transpose blocksparsematrix.hpp:224-248 + Matrix::add_transpose
 * matrix.hpp:179-187 */
int ob_add_transpose(ob_bsm *m, const ob_bsm *rhs) {
    if (m->nrb != rhs->ncb || m->ncb != rhs->nrb || m->nr != rhs->nc || m->nc != rhs->nr) return OB_EDIM;
    for (size_t ib = 0; ib < m->nrb; ++ib)
        for (size_t jb = 0; jb < m->ncb; ++jb) {
            size_t rb_ = jb + ib * rhs->nrb; /* rhs.block(jb, ib) */
            if (!rhs->blk[rb_]) continue;
            size_t b = ib + jb * m->nrb;
            int rr = rhs->brows[rb_], rc = rhs->bcols[rb_];
            if (!m->blk[b]) {
                double *d = alloc_block(m, b, rc, rr);
                for (int i = 0; i < rr * rc; ++i) d[i] = 0.0;
            }
            double *d = m->blk[b];
            int nrow = m->brows[b], ncol = m->bcols[b];
            if (nrow != rc || ncol != rr) return OB_EDIM;
            for (int c = 0; c < ncol; ++c)
                for (int r = 0; r < nrow; ++r) d[r + c * nrow] = d[r + c * nrow] + rhs->blk[rb_][c + r * rr];
            m->norm[b] = nb_nrm2(nrow * ncol, d, 1);
        }
    return OB_OK;
}

/* calc_frobenius_norms blocksparsematrix.hpp:139-147 */
void ob_calc_norms(ob_bsm *m) {
    for (size_t b = 0; b < m->nrb * m->ncb; ++b)
        m->norm[b] = m->blk[b] ? nb_nrm2(m->brows[b] * m->bcols[b], m->blk[b], 1) : 0.0;
}

/* recompress blocksparsematrix.hpp:149-156 */
void ob_recompress(ob_bsm *m) {
    const double tpb = m->thresh * (double)(m->bsc * m->bsr);
    for (size_t b = 0; b < m->nrb * m->ncb; ++b)
        if (m->norm[b] < tpb) drop_block(m, b);
}

/* frobenius_norm blocksparsematrix.hpp:256-261 */
double ob_frobenius_norm(const ob_bsm *m) {
    double acc = 0.0;
    for (size_t b = 0; b < m->nrb * m->ncb; ++b) acc = m->norm[b] * m->norm[b] + acc;
    return sqrt(acc);
}

/* no_of_alloc_blocks blocksparsematrix.hpp:158-162 */
size_t ob_no_of_alloc_blocks(const ob_bsm *m) {
    size_t n = 0;
    for (size_t b = 0; b < m->nrb * m->ncb; ++b) n += (m->blk[b] && m->brows[b] * m->bcols[b] > 0);
    return n;
}

/* to_pointer / to_matrix blocksparsematrix.hpp:103-131 (absent blocks -> 0) */
void ob_to_dense(const ob_bsm *m, double *out) {
    memset(out, 0, sizeof(double) * m->nr * m->nc);
    for (size_t rcb = 0; rcb < m->nrb * m->ncb; ++rcb) {
        if (!m->blk[rcb]) continue;
        size_t cb = rcb / m->nrb, rb = rcb % m->nrb;
        int rs = m->brows[rcb];
        for (int c = 0; c < m->bcols[rcb]; ++c)
            memcpy(&out[rb * m->bsr + (cb * m->bsc + (size_t)c) * m->nr], &m->blk[rcb][(size_t)c * rs],
                   sizeof(double) * rs);
    }
}

void ob_get_mask(const ob_bsm *m, uint8_t *mask) {
    for (size_t b = 0; b < m->nrb * m->ncb; ++b) mask[b] = m->blk[b] != NULL;
}
void ob_get_norms(const ob_bsm *m, double *norms) { memcpy(norms, m->norm, sizeof(double) * m->nrb * m->ncb); }

/* dot(BSM,BSM,thresh) blocksparsematrix.hpp:263-290 with the dense block dot
 * std::inner_product (matrix.hpp:99-103), single-threaded order */
double ob_dot(const ob_bsm *a, const ob_bsm *b, double thresh) {
    const double tpb = thresh * (double)(a->bsr * a->bsc);
    double ret = 0.0;
    for (size_t ijb = 0; ijb < a->nrb * a->ncb; ++ijb) {
        size_t ib = ijb / a->ncb, jb = ijb % a->ncb;
        size_t bi = ib + jb * a->nrb;
        if (!a->blk[bi] || !b->blk[bi]) continue;
        if (a->norm[bi] * b->norm[bi] >= tpb) {
            double d = 0.0;
            for (int i = 0; i < a->brows[bi] * a->bcols[bi]; ++i) d = d + a->blk[bi][i] * b->blk[bi][i];
            ret = ret + d;
        }
    }
    return ret;
}

/* matmult(BSM) blocksparsematrix.hpp:293-414 */
int ob_matmult(ob_bsm *C, const ob_bsm *A, int tA, const ob_bsm *B, int tB, double thresh, double alpha,
               double beta, uint64_t *nsig_out) {
    if (beta == 1.0) {
    } else if (beta == 0.0) {
        ob_zero(C);
    } else {
        ob_scale(C, beta);
    }
    const size_t ni = tA ? A->nc : A->nr, nj = tB ? B->nr : B->nc;
    const size_t nk1 = tA ? A->nr : A->nc, nk2 = tB ? B->nc : B->nr;
    if (nk1 != nk2) return OB_EDIM;
    const size_t ibs = tA ? A->bsc : A->bsr, jbs = tB ? B->bsr : B->bsc;
    if (ibs != C->bsr || jbs != C->bsc || ni != C->nr || nj != C->nc) return OB_EDIM;
    const size_t kbs1 = tA ? A->bsr : A->bsc, kbs2 = tB ? B->bsc : B->bsr;
    if (kbs1 != kbs2) return OB_EDIM;
    const size_t kbs = kbs1;
    const size_t nib = ceil_div(ni, ibs), njb = ceil_div(nj, jbs), nkb = ceil_div(nk1, kbs);
    const size_t sbs = 512;
    const size_t nib_s = ceil_div(sbs, ibs), njb_s = ceil_div(sbs, jbs), nkb_s = ceil_div(sbs, kbs);
    const size_t nibs = ceil_div(nib, nib_s), njbs = ceil_div(njb, njb_s), nkbs = ceil_div(nkb, nkb_s);
    const double tpb = thresh * (double)(ibs * jbs * kbs);
    uint64_t nsig = 0;
#pragma omp parallel for schedule(dynamic) reduction(+ : nsig)
    for (size_t ijbs = 0; ijbs < nibs * njbs; ++ijbs) {
        size_t jbs_ = ijbs / nibs, ibs_ = ijbs % nibs;
        size_t jb0 = jbs_ * njb_s, jb1 = (jbs_ + 1) * njb_s < njb ? (jbs_ + 1) * njb_s : njb;
        size_t ib0 = ibs_ * nib_s, ib1 = (ibs_ + 1) * nib_s < nib ? (ibs_ + 1) * nib_s : nib;
        for (size_t kbs_ = 0; kbs_ < nkbs; ++kbs_) {
            size_t kb0 = kbs_ * nkb_s, kb1 = (kbs_ + 1) * nkb_s < nkb ? (kbs_ + 1) * nkb_s : nkb;
            for (size_t ib = ib0; ib < ib1; ++ib)
                for (size_t jb = jb0; jb < jb1; ++jb)
                    for (size_t kb = kb0; kb < kb1; ++kb) {
                        size_t ai = tA ? kb + ib * A->nrb : ib + kb * A->nrb;
                        size_t bi = tB ? jb + kb * B->nrb : kb + jb * B->nrb;
                        size_t ci = ib + jb * C->nrb;
                        if (!A->blk[ai] || !B->blk[bi]) continue;
                        int ar = A->brows[ai], ac = A->bcols[ai], br = B->brows[bi], bc = B->bcols[bi];
                        if (ar * ac == 0 || br * bc == 0) continue;
                        int ni_act = tA ? ac : ar, nj_act = tB ? br : bc, nk_act = tA ? ar : ac;
                        double est = A->norm[ai] * B->norm[bi];
                        if (est >= tpb) {
                            int exists = C->blk[ci] != NULL;
                            if (!exists) {
                                alloc_block(C, ci, ni_act, nj_act);
                                C->norm[ci] = 0.0;
                            }
                            nsig++;
                            nb_dgemm(tA, tB, C->brows[ci], C->bcols[ci], nk_act, alpha, A->blk[ai], ar, B->blk[bi], br,
                                     exists ? 1.0 : 0.0, C->blk[ci], C->brows[ci]);
                        }
                    }
        }
    }
    if (nsig_out) *nsig_out = nsig;
    return OB_OK;
}

/* ---------------------------------------------------------------------- */
/* Hybrid Strassen-Winograd / sparse recursion (strassen.hpp)               */
/* ---------------------------------------------------------------------- */

static const double strassen_fac[20] = {10, 10, 10, 25, 35, 35, 35, 35, 35, 35,
                                        35, 35, 35, 35, 35, 35, 35, 35, 35, 35}; /* strassen.hpp:582 */

static size_t ijk3(size_t i, size_t j, size_t k, size_t di, size_t dj) { return i + j * di + k * di * dj; }

typedef struct {
    int n_levels;
    uint8_t **tree;     /* per level */
    size_t *tree_len;   /* per level */
    uint64_t *flops;    /* per level 0..L */
} ob_tree;

static void tree_free(ob_tree *t) {
    for (int l = 0; l < t->n_levels; ++l) free(t->tree[l]);
    free(t->tree);
    free(t->tree_len);
    free(t->flops);
}

/* matmult_strassen_dryrun strassen.hpp:511-679 */
static int dryrun(const ob_bsm *A, const ob_bsm *B, double tpb, ob_tree *out) {
    const size_t ni = A->nr, nj = B->nc, nk = A->nc;
    if (nk != B->nr) return OB_EDIM;
    const size_t ibs = A->bsr, jbs = B->bsc, kbs = A->bsc;
    if (kbs != B->bsr) return OB_EDIM;
    const size_t nib = ceil_div(ni, ibs), njb = ceil_div(nj, jbs), nkb = ceil_div(nk, kbs);
    if (ni != nj || ni != nk || nib != njb || nib != nkb) return OB_EDIM;
    const size_t max_level = (size_t)log2((double)nib + 0.5);
    uint64_t **nfl = (uint64_t **)calloc(max_level + 1, sizeof(uint64_t *));
    out->n_levels = (int)max_level;
    out->tree = (uint8_t **)calloc(max_level ? max_level : 1, sizeof(uint8_t *));
    out->tree_len = (size_t *)calloc(max_level ? max_level : 1, sizeof(size_t));
    out->flops = (uint64_t *)calloc(max_level + 1, sizeof(uint64_t));
    nfl[0] = (uint64_t *)calloc(nib * njb * nkb ? nib * njb * nkb : 1, sizeof(uint64_t));
    for (size_t x = 0; x < nib * njb * nkb; ++x) {
        size_t ib = x % nib, jb = (x / nib) % njb, kb = x / (nib * njb);
        size_t ai = ib + kb * A->nrb, bi = kb + jb * B->nrb;
        double est = A->norm[ai] * B->norm[bi];
        uint64_t f = 2ull * (uint64_t)A->brows[ai] * (uint64_t)B->bcols[bi] * (uint64_t)A->bcols[ai];
        nfl[0][ijk3(ib, jb, kb, nib, njb)] = (est >= tpb ? 1ull : 0ull) * f;
    }
    for (size_t x = 0; x < nib * njb * nkb; ++x) out->flops[0] += nfl[0][x];
    const uint64_t max_mult = 2ull * ibs * jbs * kbs, max_add = ibs * jbs;
    for (size_t level = 0; level < max_level; ++level) {
        const size_t psb = (size_t)exp2((double)level), sb = (size_t)exp2((double)(level + 1));
        const uint64_t c_mult = (uint64_t)round(pow(7.0, (double)(level + 1))) * max_mult;
        const uint64_t c_add = (uint64_t)(15e0 * strassen_fac[level] * pow(4.0, (double)(level + 1)) * (double)max_add);
        const uint64_t cost = c_mult + c_add;
        const size_t nsi = ceil_div(nib, sb), nsj = ceil_div(njb, sb), nsk = ceil_div(nkb, sb);
        const size_t pni = ceil_div(nib, psb), pnj = ceil_div(njb, psb);
        nfl[level + 1] = (uint64_t *)calloc(nsi * nsj * nsk, sizeof(uint64_t));
        out->tree[level] = (uint8_t *)calloc(nsi * nsj * nsk, 1);
        out->tree_len[level] = nsi * nsj * nsk;
        for (size_t s = 0; s < nsi * nsj * nsk; ++s) {
            size_t si = s % nsi, sj = (s / nsi) % nsj, sk = s / (nsi * nsj);
            size_t ib0 = si * sb, jb0 = sj * sb, kb0 = sk * sb;
            size_t ib1 = ib0 + sb < nib ? ib0 + sb : nib, jb1 = jb0 + sb < njb ? jb0 + sb : njb,
                   kb1 = kb0 + sb < nkb ? kb0 + sb : nkb;
            size_t i1 = ib1 * ibs < ni ? ib1 * ibs : ni, j1 = jb1 * jbs < nj ? jb1 * jbs : nj,
                   k1 = kb1 * kbs < nk ? kb1 * kbs : nk;
            int edge = (i1 - ib0 * ibs) != ibs * sb || (j1 - jb0 * jbs) != jbs * sb || (k1 - kb0 * kbs) != kbs * sb;
            size_t isub = ceil_div(ib1 - ib0, psb), jsub = ceil_div(jb1 - jb0, psb), ksub = ceil_div(kb1 - kb0, psb);
            uint64_t nf = 0;
            for (size_t a = 0; a < isub; ++a)
                for (size_t b = 0; b < jsub; ++b)
                    for (size_t c = 0; c < ksub; ++c) nf += nfl[level][ijk3(2 * si + a, 2 * sj + b, 2 * sk + c, pni, pnj)];
            int go = (nf >= cost) && !edge;
            out->tree[level][ijk3(si, sj, sk, nsi, nsj)] = (uint8_t)go;
            nfl[level + 1][ijk3(si, sj, sk, nsi, nsj)] = go ? cost : nf;
        }
        for (size_t s = 0; s < nsi * nsj * nsk; ++s) out->flops[level + 1] += nfl[level + 1][s];
    }
    for (size_t l = 0; l <= max_level; ++l) free(nfl[l]);
    free(nfl);
    return OB_OK;
}

int ob_strassen_dryrun(const ob_bsm *A, const ob_bsm *B, double tpb, int *n_levels, uint8_t *tree_out,
                       size_t tree_cap, uint64_t *flops_per_level) {
    ob_tree t;
    int st = dryrun(A, B, tpb, &t);
    if (st) return st;
    *n_levels = t.n_levels;
    size_t off = 0;
    for (int l = 0; l < t.n_levels; ++l) {
        if (tree_out) {
            if (off + t.tree_len[l] > tree_cap) {
                tree_free(&t);
                return OB_EPRECOND;
            }
            memcpy(tree_out + off, t.tree[l], t.tree_len[l]);
        }
        off += t.tree_len[l];
    }
    if (flops_per_level)
        for (int l = 0; l <= t.n_levels; ++l) flops_per_level[l] = t.flops[l];
    tree_free(&t);
    return OB_OK;
}

/* A grid of square bs x bs blocks: an array of block pointers with a stride
 * (ConstBlockGrid / OwnedBlockGrid strassen.hpp:57-118). */
typedef struct {
    double **p;
    size_t nrb, ncb, stride;
} grid;

static double *G(const grid *g, size_t r, size_t c) { return g->p[r + c * g->stride]; }
static grid quad(const grid *g, size_t r0, size_t c0, size_t hr, size_t hc) {
    grid q = {g->p + r0 + c0 * g->stride, hr, hc, g->stride};
    return q;
}
static grid owned(size_t nrb, size_t ncb, size_t bs2, int zero) {
    grid g;
    g.nrb = nrb;
    g.ncb = ncb;
    g.stride = nrb;
    g.p = (double **)malloc(sizeof(double *) * (nrb * ncb ? nrb * ncb : 1));
    for (size_t i = 0; i < nrb * ncb; ++i) g.p[i] = zero ? (double *)calloc(bs2, sizeof(double)) : (double *)malloc(bs2 * sizeof(double));
    return g;
}
static void owned_free(grid *g) {
    for (size_t i = 0; i < g->nrb * g->ncb; ++i) free(g->p[i]);
    free(g->p);
}

typedef struct {
    size_t bs, min_size;
} sctx;

static void leaf_gemm(const sctx *s, double *c, const double *a, const double *b) {
    /* gemm_block strassen.hpp:42-50 with alpha = beta = 1 */
    nb_dgemm(0, 0, (int)s->bs, (int)s->bs, (int)s->bs, 1.0, a, (int)s->bs, b, (int)s->bs, 1.0, c, (int)s->bs);
}

static void strassen_recurse(const sctx *s, grid *C00, grid *C01, grid *C10, grid *C11, const grid *a, const grid *b,
                             const grid *c, const grid *d, const grid *A, const grid *C, const grid *B, const grid *D);

/* strassen_matmult_acc strassen.hpp:296-353 */
static void matmult_acc(const sctx *s, grid *X, const grid *P, const grid *Q) {
    const size_t nrb = X->nrb, nkb = P->ncb, ncb = X->ncb;
    if (nrb == 1 && nkb == 1 && ncb == 1) {
        leaf_gemm(s, G(X, 0, 0), G(P, 0, 0), G(Q, 0, 0));
        return;
    }
    const int too_small = nrb * s->bs <= s->min_size;
    if (nrb % 2 || nkb % 2 || ncb % 2 || too_small) {
        for (size_t cb = 0; cb < ncb; ++cb)
            for (size_t rb = 0; rb < nrb; ++rb)
                for (size_t kb = 0; kb < nkb; ++kb) leaf_gemm(s, G(X, rb, cb), G(P, rb, kb), G(Q, kb, cb));
        return;
    }
    const size_t hr = nrb / 2, hk = nkb / 2, hc = ncb / 2, bs2 = s->bs * s->bs;
    grid aq = quad(P, 0, 0, hr, hk), bq = quad(P, 0, hk, hr, hk), cq = quad(P, hr, 0, hr, hk), dq = quad(P, hr, hk, hr, hk);
    grid Aq = quad(Q, 0, 0, hk, hc), Cq = quad(Q, 0, hc, hk, hc), Bq = quad(Q, hk, 0, hk, hc), Dq = quad(Q, hk, hc, hk, hc);
    grid S00 = owned(hr, hc, bs2, 1), S01 = owned(hr, hc, bs2, 1), S10 = owned(hr, hc, bs2, 1), S11 = owned(hr, hc, bs2, 1);
    strassen_recurse(s, &S00, &S01, &S10, &S11, &aq, &bq, &cq, &dq, &Aq, &Cq, &Bq, &Dq);
    for (size_t cb = 0; cb < hc; ++cb)
        for (size_t rb = 0; rb < hr; ++rb) {
            nb_daxpy((int)bs2, 1.0, G(&S00, rb, cb), 1, G(X, rb, cb), 1);
            nb_daxpy((int)bs2, 1.0, G(&S01, rb, cb), 1, G(X, rb, cb + hc), 1);
            nb_daxpy((int)bs2, 1.0, G(&S10, rb, cb), 1, G(X, rb + hr, cb), 1);
            nb_daxpy((int)bs2, 1.0, G(&S11, rb, cb), 1, G(X, rb + hr, cb + hc), 1);
        }
    owned_free(&S00);
    owned_free(&S01);
    owned_free(&S10);
    owned_free(&S11);
}

/* strassen_recurse strassen.hpp:359-405 with the fused pre-sums
 * (strassen_prepare_A_side :153-182, strassen_prepare_B_side :184-213) and
 * post-sum (strassen_post_process_C_side :215-237) */
static void strassen_recurse(const sctx *s, grid *C00, grid *C01, grid *C10, grid *C11, const grid *a, const grid *b,
                             const grid *c, const grid *d, const grid *A, const grid *C, const grid *B, const grid *D) {
    const size_t nrb = C00->nrb, nkb = a->ncb, ncb = C00->ncb, bs2 = s->bs * s->bs;
    grid na_pc = owned(nrb, nkb, bs2, 0), pc_pd = owned(nrb, nkb, bs2, 0), na_pc_pd = owned(nrb, nkb, bs2, 0),
         pa_pb_nc_nd = owned(nrb, nkb, bs2, 0);
    for (size_t cb = 0; cb < nkb; ++cb)
        for (size_t rb = 0; rb < nrb; ++rb) {
            double *o1 = G(&na_pc, rb, cb), *o2 = G(&pc_pd, rb, cb), *o3 = G(&na_pc_pd, rb, cb), *o4 = G(&pa_pb_nc_nd, rb, cb);
            const double *pa = G(a, rb, cb), *pb = G(b, rb, cb), *pc = G(c, rb, cb), *pd = G(d, rb, cb);
            for (size_t i = 0; i < bs2; ++i) {
                o1[i] = pc[i] - pa[i];
                const double v = pc[i] + pd[i];
                o2[i] = v;
                const double w = v - pa[i];
                o3[i] = w;
                o4[i] = pb[i] - w;
            }
        }
    grid pC_nD = owned(nkb, ncb, bs2, 0), nA_pC = owned(nkb, ncb, bs2, 0), pA_nC_pD = owned(nkb, ncb, bs2, 0),
         nA_pB_pC_nD = owned(nkb, ncb, bs2, 0);
    for (size_t cb = 0; cb < ncb; ++cb)
        for (size_t rb = 0; rb < nkb; ++rb) {
            double *o1 = G(&pC_nD, rb, cb), *o2 = G(&nA_pC, rb, cb), *o3 = G(&pA_nC_pD, rb, cb), *o4 = G(&nA_pB_pC_nD, rb, cb);
            const double *qA = G(A, rb, cb), *qB = G(B, rb, cb), *qC = G(C, rb, cb), *qD = G(D, rb, cb);
            for (size_t i = 0; i < bs2; ++i) {
                o1[i] = qC[i] - qD[i];
                const double v = qC[i] - qA[i];
                o2[i] = v;
                const double w = qD[i] - v;
                o3[i] = w;
                o4[i] = qB[i] - w;
            }
        }
    matmult_acc(s, C00, a, A);              /* M1 */
    matmult_acc(s, C10, &na_pc, &pC_nD);    /* M2 */
    matmult_acc(s, C01, &pc_pd, &nA_pC);    /* M3 */
    matmult_acc(s, C11, &na_pc_pd, &pA_nC_pD); /* M4 -> nw */
    for (size_t cb = 0; cb < ncb; ++cb)
        for (size_t rb = 0; rb < nrb; ++rb) {
            double *nw = G(C11, rb, cb), *c00 = G(C00, rb, cb), *c01 = G(C01, rb, cb), *c10 = G(C10, rb, cb);
            for (size_t i = 0; i < bs2; ++i) {
                const double t = nw[i] + c00[i];
                c10[i] = c10[i] + t;
                nw[i] = c01[i] + c10[i];
                c01[i] = c01[i] + t;
            }
        }
    matmult_acc(s, C01, &pa_pb_nc_nd, D);  /* M5 */
    matmult_acc(s, C10, d, &nA_pB_pC_nD);  /* M6 */
    matmult_acc(s, C00, b, B);             /* M7 */
    owned_free(&na_pc);
    owned_free(&pc_pd);
    owned_free(&na_pc_pd);
    owned_free(&pa_pb_nc_nd);
    owned_free(&pC_nD);
    owned_free(&nA_pC);
    owned_free(&pA_nC_pD);
    owned_free(&nA_pB_pC_nD);
}

typedef struct {
    ob_bsm *Cm;
    const ob_bsm *Am, *Bm;
    const ob_tree *tree;
    double tpb;
    sctx s;
    int err;
} hctx;

static grid bsm_view(const ob_bsm *M, size_t ib0, size_t jb0, size_t nrb, size_t ncb) {
    /* bsm_quadrant_view strassen.hpp:125-136 */
    grid g;
    g.nrb = nrb;
    g.ncb = ncb;
    g.stride = nrb;
    g.p = (double **)malloc(sizeof(double *) * nrb * ncb);
    for (size_t cb = 0; cb < ncb; ++cb)
        for (size_t rb = 0; rb < nrb; ++rb) g.p[rb + cb * nrb] = M->blk[(ib0 + rb) + (jb0 + cb) * M->nrb];
    return g;
}

static int view_full(const ob_bsm *M, size_t ib0, size_t jb0, size_t n, size_t bs) {
    for (size_t cb = 0; cb < n; ++cb)
        for (size_t rb = 0; rb < n; ++rb) {
            size_t b = (ib0 + rb) + (jb0 + cb) * M->nrb;
            if (!M->blk[b] || (size_t)M->brows[b] != bs || (size_t)M->bcols[b] != bs) return 0;
        }
    return 1;
}

/* hybrid_recurse strassen.hpp:418-508 */
static void hybrid(hctx *h, size_t ib0, size_t jb0, size_t kb0, size_t sb, long level) {
    const size_t nib = h->Am->nrb, njb = h->Bm->ncb, nkb = h->Am->ncb;
    if (h->err) return;
    if (level < 0) {
        if (ib0 >= nib || jb0 >= njb || kb0 >= nkb) return;
        size_t ai = ib0 + kb0 * h->Am->nrb, bi = kb0 + jb0 * h->Bm->nrb, ci = ib0 + jb0 * h->Cm->nrb;
        if (!h->Am->blk[ai] || !h->Bm->blk[bi]) return;
        if (h->Am->norm[ai] * h->Bm->norm[bi] < h->tpb) return;
        if (!h->Cm->blk[ci]) return; /* size-0 C view: BLAS no-op */
        nb_dgemm(0, 0, h->Cm->brows[ci], h->Cm->bcols[ci], h->Am->bcols[ai], 1.0, h->Am->blk[ai], h->Am->brows[ai],
                 h->Bm->blk[bi], h->Bm->brows[bi], 1.0, h->Cm->blk[ci], h->Cm->brows[ci]);
        return;
    }
    const size_t n_si = ceil_div(nib, sb), n_sj = ceil_div(njb, sb);
    const size_t si = ib0 / sb, sj = jb0 / sb, sk = kb0 / sb;
    const int go = h->tree->tree[level][ijk3(si, sj, sk, n_si, n_sj)];
    if (go) {
        const size_t hh = sb / 2, bs = h->s.bs, bs2 = bs * bs;
        if (!view_full(h->Am, ib0, kb0, sb, bs) || !view_full(h->Bm, kb0, jb0, sb, bs) ||
            !view_full(h->Cm, ib0, jb0, sb, bs)) {
            h->err = OB_EPRECOND;
            return;
        }
        grid qa = bsm_view(h->Am, ib0, kb0, hh, hh), qb = bsm_view(h->Am, ib0, kb0 + hh, hh, hh),
             qc = bsm_view(h->Am, ib0 + hh, kb0, hh, hh), qd = bsm_view(h->Am, ib0 + hh, kb0 + hh, hh, hh);
        grid qA = bsm_view(h->Bm, kb0, jb0, hh, hh), qC = bsm_view(h->Bm, kb0, jb0 + hh, hh, hh),
             qB = bsm_view(h->Bm, kb0 + hh, jb0, hh, hh), qD = bsm_view(h->Bm, kb0 + hh, jb0 + hh, hh, hh);
        grid S00 = owned(hh, hh, bs2, 1), S01 = owned(hh, hh, bs2, 1), S10 = owned(hh, hh, bs2, 1), S11 = owned(hh, hh, bs2, 1);
        strassen_recurse(&h->s, &S00, &S01, &S10, &S11, &qa, &qb, &qc, &qd, &qA, &qC, &qB, &qD);
        /* accumulate_into_bsm strassen.hpp:249-256 */
        grid *Ss[4] = {&S00, &S01, &S10, &S11};
        size_t oi[4] = {ib0, ib0, ib0 + hh, ib0 + hh}, oj[4] = {jb0, jb0 + hh, jb0, jb0 + hh};
        for (int q = 0; q < 4; ++q)
            for (size_t cb = 0; cb < hh; ++cb)
                for (size_t rb = 0; rb < hh; ++rb)
                    nb_daxpy((int)bs2, 1.0, G(Ss[q], rb, cb), 1, h->Cm->blk[(oi[q] + rb) + (oj[q] + cb) * h->Cm->nrb], 1);
        free(qa.p); free(qb.p); free(qc.p); free(qd.p);
        free(qA.p); free(qC.p); free(qB.p); free(qD.p);
        owned_free(&S00); owned_free(&S01); owned_free(&S10); owned_free(&S11);
    } else {
        const size_t hh = sb / 2;
        for (size_t dj = 0; dj < 2; ++dj) {
            size_t cj = jb0 + dj * hh;
            if (cj >= njb) continue;
            for (size_t di = 0; di < 2; ++di) {
                size_t ci = ib0 + di * hh;
                if (ci >= nib) continue;
                for (size_t dk = 0; dk < 2; ++dk) {
                    size_t ck = kb0 + dk * hh;
                    if (ck >= nkb) continue;
                    hybrid(h, ci, cj, ck, hh, level - 1);
                }
            }
        }
    }
}

/* matmult_strassen_sparse strassen.hpp:687-753 (no transposes, alpha = 1,
 * beta ignored: C must be pre-filled) */
int ob_matmult_strassen_sparse(ob_bsm *C, const ob_bsm *A, const ob_bsm *B, double thresh, size_t min_size) {
    const size_t nib = A->nrb, njb = B->ncb, nkb = A->ncb;
    if (nkb != B->nrb || nib != C->nrb || njb != C->ncb || nib != njb || nib != nkb) return OB_EDIM;
    if (A->bsr != A->bsc || A->bsr != B->bsc || B->bsr != B->bsc) return OB_EDIM;
    const double tpb = thresh * (double)(A->bsr * B->bsc * A->bsc);
    ob_tree t;
    int st = dryrun(A, B, tpb, &t);
    if (st) return st;
    const size_t max_level = (size_t)t.n_levels;
    const long top_level = (long)max_level - 1;
    const size_t top_sb = (size_t)exp2((double)max_level);
    const size_t nsi = ceil_div(nib, top_sb), nsj = ceil_div(njb, top_sb), nsk = ceil_div(nkb, top_sb);
    hctx h = {C, A, B, &t, tpb, {A->bsr, min_size}, 0};
    for (size_t sk = 0; sk < nsk; ++sk)
        for (size_t sj = 0; sj < nsj; ++sj)
            for (size_t si = 0; si < nsi; ++si) hybrid(&h, si * top_sb, sj * top_sb, sk * top_sb, top_sb, top_level);
    tree_free(&t);
    return h.err;
}

/* ---------------------------------------------------------------------- */
/* Drivers                                                                  */
/* ---------------------------------------------------------------------- */

/* libgomp schedule(static) without a chunk size: thread t of T gets a
 * contiguous range, the first n%T threads one element more */
static void static_range(size_t n, int T, int t, size_t *lo, size_t *hi) {
    size_t q = n / (size_t)T, r = n % (size_t)T;
    size_t tt = (size_t)t;
    *lo = tt * q + (tt < r ? tt : r);
    *hi = *lo + q + (tt < r ? 1 : 0);
}

/* decompress_integrals occ_ri_k_step.cpp:133-146 */
static int decompress(double *U, size_t n_bf, size_t P, const double *ints, size_t n_vec2, const uint64_t *keys) {
    for (size_t v = 0; v < n_vec2; ++v) {
        if (keys[v] >= n_bf * n_bf) return OB_EPRECOND;
        U[keys[v]] = ints[v + P * n_vec2];
    }
    return OB_OK;
}

/* block-sparse occ-RI-K occ_ri_k_step.cpp:83-130.  Partitions run as an
 * OpenMP team (one partial K each, :90-118); the partials are then added in
 * partition order, which fixes the order the reference's critical section
 * (:119-122) leaves open. */
int ob_rik_occ_step(size_t n_bf, size_t n_aux, size_t n_occ, size_t n_vec2, const double *ints, const uint64_t *keys,
                    const double *c_occ, size_t bs, double thresh, int n_part, double *k_out) {
    if (n_part < 1) return OB_EPRECOND;
    for (size_t v = 0; v < n_vec2; ++v)
        if (keys[v] >= n_bf * n_bf) return OB_EPRECOND;
    ob_bsm *K = ob_create(n_bf, n_occ, bs, bs, 0.0);
    ob_fill(K, 0.0);
    ob_bsm *Cb = ob_create(n_bf, n_occ, bs, bs, 0.0);
    ob_copy_from_dense(Cb, c_occ);
    ob_bsm **Kpart = (ob_bsm **)calloc((size_t)n_part, sizeof(ob_bsm *));
    int st = OB_OK;
#pragma omp parallel for schedule(dynamic, 1) reduction(| : st)
    for (int t = 0; t < n_part; ++t) {
        double *U = (double *)calloc(n_bf * n_bf, sizeof(double));
        ob_bsm *Ub = ob_create(n_bf, n_bf, bs, bs, 1e-20);
        ob_bsm *mui = ob_create(n_bf, n_occ, bs, bs, 0.0);
        ob_bsm *ij = ob_create(n_occ, n_occ, bs, bs, 0.0);
        ob_bsm *ijs = ob_create(n_occ, n_occ, bs, bs, 0.0);
        ob_bsm *Ks = ob_create(n_bf, n_occ, bs, bs, 0.0);
        ob_fill(Ks, 0.0);
        size_t lo, hi;
        static_range(n_aux, n_part, t, &lo, &hi);
        int lst = OB_OK;
        for (size_t P = lo; P < hi && !lst; ++P) {
            decompress(U, n_bf, P, ints, n_vec2, keys);
            ob_copy_from_dense(Ub, U);
            lst = ob_matmult(mui, Ub, 0, Cb, 0, thresh, 1.0, 0.0, NULL);
            if (lst) break;
            ob_calc_norms(mui);
            lst = ob_matmult(ij, Cb, 1, mui, 0, thresh, 1.0, 0.0, NULL);
            if (lst) break;
            ob_copy(ijs, ij);
            lst = ob_add_transpose(ijs, ij);
            if (lst) break;
            lst = ob_matmult(Ks, mui, 0, ijs, 0, thresh, 1.0, 1.0, NULL);
        }
        Kpart[t] = Ks;
        st |= lst;
        free(U);
        ob_free(Ub);
        ob_free(mui);
        ob_free(ij);
        ob_free(ijs);
    }
    for (int t = 0; t < n_part && !st; ++t) st = ob_add(K, Kpart[t]);
    for (int t = 0; t < n_part; ++t) ob_free(Kpart[t]);
    free(Kpart);
    if (!st) ob_to_dense(K, k_out);
    ob_free(K);
    ob_free(Cb);
    return st;
}

/* Symmetric exchange matrix K_mn = sum_{P,i} mui_P(m,i) mui_P(n,i), N_bf x N_bf.
 * The reference computes only K_{mu j} (occ_ri_k_step.cpp:83-130); this is the
 * same pipeline's adjacent contraction written with its own operations: mui_P
 * exactly as the occ step builds it (:102-108), then per P
 * matmult(Kmn_sub, mui_P, N, mui_P, T, thresh, 1, 1) the way :116 adds
 * mui_P ijs_P into K_sub, and the partition partials added in order (:119-122). */
int ob_rik_kmn_step(size_t n_bf, size_t n_aux, size_t n_occ, size_t n_vec2, const double *ints, const uint64_t *keys,
                    const double *c_occ, size_t bs, double thresh, int n_part, double *kmn_out) {
    if (n_part < 1) return OB_EPRECOND;
    for (size_t v = 0; v < n_vec2; ++v)
        if (keys[v] >= n_bf * n_bf) return OB_EPRECOND;
    ob_bsm *K = ob_create(n_bf, n_bf, bs, bs, 0.0);
    ob_fill(K, 0.0);
    ob_bsm *Cb = ob_create(n_bf, n_occ, bs, bs, 0.0);
    ob_copy_from_dense(Cb, c_occ);
    ob_bsm **Kpart = (ob_bsm **)calloc((size_t)n_part, sizeof(ob_bsm *));
    int st = OB_OK;
#pragma omp parallel for schedule(dynamic, 1) reduction(| : st)
    for (int t = 0; t < n_part; ++t) {
        double *U = (double *)calloc(n_bf * n_bf, sizeof(double));
        ob_bsm *Ub = ob_create(n_bf, n_bf, bs, bs, 1e-20);
        ob_bsm *mui = ob_create(n_bf, n_occ, bs, bs, 0.0);
        ob_bsm *Ks = ob_create(n_bf, n_bf, bs, bs, 0.0);
        ob_fill(Ks, 0.0);
        size_t lo, hi;
        static_range(n_aux, n_part, t, &lo, &hi);
        int lst = OB_OK;
        for (size_t P = lo; P < hi && !lst; ++P) {
            decompress(U, n_bf, P, ints, n_vec2, keys);
            ob_copy_from_dense(Ub, U);
            lst = ob_matmult(mui, Ub, 0, Cb, 0, thresh, 1.0, 0.0, NULL);
            if (lst) break;
            ob_calc_norms(mui);
            lst = ob_matmult(Ks, mui, 0, mui, 1, thresh, 1.0, 1.0, NULL);
        }
        Kpart[t] = Ks;
        st |= lst;
        free(U);
        ob_free(Ub);
        ob_free(mui);
    }
    for (int t = 0; t < n_part && !st; ++t) st = ob_add(K, Kpart[t]);
    for (int t = 0; t < n_part; ++t) ob_free(Kpart[t]);
    free(Kpart);
    if (!st) ob_to_dense(K, kmn_out);
    ob_free(K);
    ob_free(Cb);
    return st;
}

/* dense occ-RI-K occ_ri_k_step.cpp:39-77 */
int ob_rik_occ_dense(size_t n_bf, size_t n_aux, size_t n_occ, size_t n_vec2, const double *ints, const uint64_t *keys,
                     const double *c_occ, int n_part, double *k_out) {
    if (n_part < 1) return OB_EPRECOND;
    double *U = (double *)malloc(sizeof(double) * n_bf * n_bf);
    double *mui = (double *)malloc(sizeof(double) * n_bf * n_occ);
    double *ij = (double *)malloc(sizeof(double) * n_occ * n_occ);
    double *ijs = (double *)malloc(sizeof(double) * n_occ * n_occ);
    double *Ks = (double *)malloc(sizeof(double) * n_bf * n_occ);
    memset(k_out, 0, sizeof(double) * n_bf * n_occ);
    int st = OB_OK;
    for (int t = 0; t < n_part && !st; ++t) {
        memset(U, 0, sizeof(double) * n_bf * n_bf);
        memset(Ks, 0, sizeof(double) * n_bf * n_occ);
        size_t lo, hi;
        static_range(n_aux, n_part, t, &lo, &hi);
        for (size_t P = lo; P < hi; ++P) {
            st = decompress(U, n_bf, P, ints, n_vec2, keys);
            if (st) break;
            nb_dgemm(0, 0, (int)n_bf, (int)n_occ, (int)n_bf, 1.0, U, (int)n_bf, c_occ, (int)n_bf, 0.0, mui, (int)n_bf);
            nb_dgemm(1, 0, (int)n_occ, (int)n_occ, (int)n_bf, 1.0, c_occ, (int)n_bf, mui, (int)n_bf, 0.0, ij, (int)n_occ);
            memcpy(ijs, ij, sizeof(double) * n_occ * n_occ);
            for (size_t c = 0; c < n_occ; ++c)
                for (size_t r = 0; r < n_occ; ++r) ijs[r + c * n_occ] = ijs[r + c * n_occ] + ij[c + r * n_occ];
            nb_dgemm(0, 0, (int)n_bf, (int)n_occ, (int)n_occ, 1.0, mui, (int)n_bf, ijs, (int)n_occ, 1.0, Ks, (int)n_bf);
        }
        nb_daxpy((int)(n_bf * n_occ), 1.0, Ks, 1, k_out, 1);
    }
    free(U);
    free(mui);
    free(ij);
    free(ijs);
    free(Ks);
    return st;
}

/* 3c_2c_transform.cpp:44-57: out = X_bsm * V_bsm with both inputs built at
 * threshold 0 and the output pre-filled with zeros (beta = 1) */
int ob_3c2c_transform(size_t n_vec2, size_t n_aux, const double *ints_3c, const double *v_m12, size_t bs, double thresh,
                      double *out) {
    ob_bsm *X = ob_create(n_vec2, n_aux, bs, bs, 0.0), *V = ob_create(n_aux, n_aux, bs, bs, 0.0),
           *O = ob_create(n_vec2, n_aux, bs, bs, 0.0);
    ob_copy_from_dense(X, ints_3c);
    ob_copy_from_dense(V, v_m12);
    ob_fill(O, 0.0);
    int st = ob_matmult(O, X, 0, V, 0, thresh, 1.0, 1.0, NULL);
    if (!st) ob_to_dense(O, out);
    ob_free(X);
    ob_free(V);
    ob_free(O);
    return st;
}
