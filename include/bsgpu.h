/*
 * bsgpu -- GB300 (sm_103a) block-sparse GEMM, hybrid Strassen-Winograd /
 * sparse recursion and RI-K exchange step behind a C ABI.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, returns a
 * bsg_status (0 = success) and leaves a message in bsg_last_error() on
 * failure.  Where the reference asserts or calls exit(1) (matrix.hpp:63-74,
 * blocksparsematrix.hpp:308-338, strassen.hpp:693-705) these functions
 * return BSG_ERR_ARG or BSG_ERR_PRECOND instead and launch nothing.
 *
 * Arithmetic: the FP64 form performs, for every output element, the same
 * sequence of IEEE-754 operations as the reference linked against the
 * deterministic BLAS definition (dgemm: for every element an fma chain over k
 * in order from zero, then C = alpha*t + beta*C; nrm2: 32 lane-strided fma
 * chains combined by a shuffle tree), so its results, block masks and cached
 * norms are bit-identical to that reference.
 *
 * Threading: a bsg_ctx owns one CUDA stream; calls on one context are
 * ordered on that stream.  Host threads may call concurrently only on
 * distinct contexts (and matrices belonging to them).
 */
#ifndef BSGPU_H
#define BSGPU_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int bsg_status;
enum {
    BSG_OK = 0,
    BSG_ERR_ARG = 1,         /* bad argument or dimension mismatch */
    BSG_ERR_PRECOND = 2,     /* a precondition the reference asserts on */
    BSG_ERR_CUDA = 3,        /* CUDA runtime error (message has details) */
    BSG_ERR_NOMEM = 4,       /* device or host allocation failed */
    BSG_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up */
    BSG_ERR_UNSUPPORTED = 6  /* configuration outside what is implemented */
};

enum { BSG_HOST = 0, BSG_DEVICE = 1 }; /* where a buffer lives */

/* arithmetic form of a product */
enum {
    BSG_FORM_FP64 = 0,  /* plain FP64, bit-identical to the reference */
    BSG_FORM_OZAKI = 1  /* bf16 digit slices on tcgen05, exact fp32 partial sums, fp64 combine */
};

typedef struct bsg_ctx_s *bsg_ctx;
typedef struct bsg_pool_s *bsg_pool;
typedef struct bsg_bsm_s *bsg_bsm;
typedef struct bsg_sched_s *bsg_sched;
typedef struct bsg_batch_plan_s *bsg_batch_plan;

const char *bsg_last_error(void);
int bsg_version(void);

/* ---- context (device + stream; no counterpart in the reference, which runs
 *      on the host: every call below takes the context or an object made on it) ---- */
bsg_status bsg_ctx_create(int device, void *cuda_stream, bsg_ctx *out);
bsg_status bsg_ctx_destroy(bsg_ctx ctx);
bsg_status bsg_ctx_sync(bsg_ctx ctx);
/* number of kernels this context has launched so far */
bsg_status bsg_ctx_launch_count(bsg_ctx ctx, uint64_t *out);
/* Timing of the tensor-core (Ozaki form) GEMM launches with CUDA events on
 * the context's stream: enable/disable (resets the totals), then read the
 * launch count, total milliseconds and the unpadded block-product
 * multiply-adds they performed (FP64-equivalent; x digit products for bf16). */
bsg_status bsg_ctx_set_timing(bsg_ctx ctx, int on);
bsg_status bsg_ctx_gemm_timing(bsg_ctx ctx, uint64_t *launches, double *ms, double *useful_macs);
/* Pipeline stall breakdown of the same launches (SM clock cycles summed over
 * CTAs; collected only while timing is on): [0] MMA issuer waiting for
 * operand stages, [1] MMA issuer waiting for a drained accumulator, [2] MMA
 * issuer lifetime, [3] producer waiting for a free stage, [4] epilogue
 * waiting for a finished chain, [5] epilogue draining TMEM, [6] epilogue
 * writing output blocks, [7] operand stages consumed, [8] MMA instructions
 * issued, [9] k steps copied, [10] (live slot, live N-side block) pairs in
 * those steps, [11] slots x N-side blocks of those steps (the capacity). */
bsg_status bsg_ctx_gemm_stalls(bsg_ctx ctx, uint64_t out[12]);

/* ---- block pool: BlockMemoryPool<double> (blockallocator.h:8-25,
 *      blockallocator.hpp:7-56).  Device slabs grow geometrically from 16 MB
 *      to 1 GB; blocks are handed out from a free list.  A pool is shared by
 *      every matrix created on it and lives until its last user is gone. ---- */
bsg_status bsg_pool_create(bsg_ctx ctx, size_t block_elems, bsg_pool *out);
bsg_status bsg_pool_release(bsg_pool pool);                          /* drop the caller's reference */
bsg_status bsg_pool_adjust_blocksize(bsg_pool pool, size_t block_elems); /* blockallocator.hpp:51-56 */
bsg_status bsg_pool_release_all_memory(bsg_pool pool);               /* blockallocator.hpp:58-62 */
bsg_status bsg_pool_stats(bsg_pool pool, size_t *blocks_total, size_t *blocks_free, size_t *bytes);

/* ---- BlockSparseMatrix<double> (blocksparsematrix.h:19-93) ---- */
/* BlockSparseMatrix(nr, nc, bsr, bsc, thresh[, pool]) blocksparsematrix.hpp:5-15;
 * pool may be NULL (a fresh pool of bsr*bsc-element blocks, :15) */
bsg_status bsg_bsm_create(bsg_ctx ctx, size_t nr, size_t nc, size_t bsr, size_t bsc, double thresh, bsg_pool pool,
                          bsg_bsm *out);
bsg_status bsg_bsm_destroy(bsg_bsm m); /* end of the BlockSparseMatrix's life; its blocks go back to its pool */
/* dims[0..5] = nr, nc, bsr, bsc, nrb, ncb; *thresh = the per-element threshold:
 * nrow/ncol/max_blocksize_row/max_blocksize_col/nrowblocks/ncolblocks/thresh
 * accessors, blocksparsematrix.h:49-55 */
bsg_status bsg_bsm_info(bsg_bsm m, size_t dims[6], double *thresh);
bsg_status bsg_bsm_pool(bsg_bsm m, bsg_pool *out); /* mem_pool_ptr() blocksparsematrix.h:81 */
/* copy assignment: blocks and cached norms (used as `ijs = ij`, occ_ri_k_step.cpp:112) */
bsg_status bsg_bsm_assign(bsg_bsm dst, bsg_bsm src);
/* copy_from_input_array / copy_from_input_matrix blocksparsematrix.hpp:35-69:
 * column-major nr x nc input; blocks with norm < thresh*bsr*bsc are dropped */
bsg_status bsg_bsm_copy_from_dense(bsg_bsm m, const double *in, int where);
bsg_status bsg_bsm_fill(bsg_bsm m, double val);  /* fill_with_values :84-101 */
bsg_status bsg_bsm_zero(bsg_bsm m);              /* zero :79-82 */
bsg_status bsg_bsm_scale(bsg_bsm m, double s);   /* scale / operator*= :71-77,250-254 */
bsg_status bsg_bsm_add(bsg_bsm m, bsg_bsm rhs);  /* operator+= :170-194 */
bsg_status bsg_bsm_sub(bsg_bsm m, bsg_bsm rhs);  /* operator-= :196-221 */
bsg_status bsg_bsm_add_transpose(bsg_bsm m, bsg_bsm rhs); /* add_transpose :224-248 */
bsg_status bsg_bsm_calc_norms(bsg_bsm m);        /* calc_frobenius_norms :139-147 */
bsg_status bsg_bsm_recompress(bsg_bsm m);        /* recompress :149-156 */
bsg_status bsg_bsm_frobenius_norm(bsg_bsm m, double *out);       /* frobenius_norm :256-261 */
bsg_status bsg_bsm_no_of_alloc_blocks(bsg_bsm m, size_t *out);   /* no_of_alloc_blocks :158-162 */
bsg_status bsg_bsm_calc_alloc_dim(bsg_bsm m, size_t *out);       /* calc_alloc_dim :164-168 */
/* to_pointer / to_matrix :103-131 (absent blocks read as zero) */
bsg_status bsg_bsm_to_dense(bsg_bsm m, double *out, int where);
/* block presence (1/0) and cached norms, block (r,c) at index r + c*nrb (the
 * reference's block(r, c) storage order, blocksparsematrix.h:71-72, and each
 * block's frobenius_norm(), matrix.h:52-53; for mask parity tests) */
bsg_status bsg_bsm_get_mask(bsg_bsm m, uint8_t *mask_host);
bsg_status bsg_bsm_get_norms(bsg_bsm m, double *norms_host);

/* dot(BSM, BSM, thresh) blocksparsematrix.hpp:263-290 */
bsg_status bsg_dot(bsg_bsm a, bsg_bsm b, double thresh, double *out);

/* matmult(C, A, tA, B, tB, thresh, alpha, beta) blocksparsematrix.hpp:293-414:
 * C = alpha*op(A)*op(B) + beta*C over block triples with
 * ||A_ik||*||B_kj|| >= thresh*bs_i*bs_j*bs_k.  *nsig_out (may be NULL)
 * receives the number of surviving block products. */
bsg_status bsg_matmult(bsg_bsm C, bsg_bsm A, int tA, bsg_bsm B, int tB, double thresh, double alpha, double beta,
                       uint64_t *nsig_out);
/* the same product in a chosen arithmetic form (BSG_FORM_OZAKI: n_digits
 * bf16 slices per operand, 2..8, 0 = 5 where two pipeline stages fit shared
 * memory, else 4).  Screening uses the operands' cached FP64 norms in both
 * forms, so this product's mask and surviving pairs equal the FP64 form's for
 * the same operands.  A later screen on norms of a result computed in the
 * mixed form (RI-K's mui_P and ijs_P) can differ from the FP64 form's for
 * blocks whose norm product lies within the result's error of the threshold. */
bsg_status bsg_matmult_form(bsg_bsm C, bsg_bsm A, int tA, bsg_bsm B, int tB, double thresh, double alpha,
                            double beta, int form, int n_digits, uint64_t *nsig_out);

/* ---- hybrid Strassen-Winograd / sparse recursion (strassen.hpp) ---- */
/* matmult_strassen_dryrun strassen.hpp:511-679: decision-tree bits of levels
 * 0..L-1 concatenated into tree_host (level l holds ceil(nb/2^(l+1))^3
 * entries, index si + sj*n + sk*n*n), flops_per_level[0..L] */
bsg_status bsg_strassen_dryrun(bsg_bsm A, bsg_bsm B, double thresh_per_block, int *n_levels, uint8_t *tree_host,
                               size_t tree_cap, uint64_t *flops_per_level);
/* matmult_strassen_sparse strassen.hpp:687-753 (square, no transposes,
 * alpha = 1, beta ignored: C must be pre-filled, as main.cpp:57 does);
 * min_size_for_strassen is the reference's global knob (main.cpp:9) */
bsg_status bsg_matmult_strassen_sparse(bsg_bsm C, bsg_bsm A, int tA, bsg_bsm B, int tB, double thresh,
                                       double alpha, double beta, size_t min_size_for_strassen);
bsg_status bsg_matmult_strassen_sparse_form(bsg_bsm C, bsg_bsm A, bsg_bsm B, double thresh,
                                            size_t min_size_for_strassen, int form, int n_digits);

/* ---- batched products (many independent screened products of mixed sizes
 *      in one call; no single counterpart in the reference, which calls
 *      matmult once per product) ----
 * C_i = alpha A_i B_i + beta C_i for i < n, each with matmult's semantics
 * (no transposes), any sizes and block sizes.  Mixed form: products are
 * grouped by block sizes, and ONE persistent tensor-core launch runs the
 * tiles of every group (up to 8 groups per launch), each tile in its group's
 * geometry; the tile height per group shape comes from an autotuner (timed
 * on first use, group by group, cached in the context).  nsig_total (may be
 * NULL) receives the surviving block triples of all products. */
bsg_status bsg_matmult_batched(size_t n, const bsg_bsm *C, const bsg_bsm *A, const bsg_bsm *B, double thresh,
                               double alpha, double beta, int form, int n_digits, uint64_t *nsig_total);
/* A batch (mixed form, beta 0) captured as a CUDA graph: creating the plan
 * screens, allocates the C blocks, tunes and runs the batch once; each run
 * replays the device work (digit images, step lists, the persistent launches)
 * from the operands' current values.  Valid while the operands' block
 * structure and cached norms are those the plan was made with and the C
 * blocks stay allocated (no zero / recompress / destroy of C in between). */
bsg_status bsg_batched_plan_create(size_t n, const bsg_bsm *C, const bsg_bsm *A, const bsg_bsm *B, double thresh,
                                   double alpha, int n_digits, bsg_batch_plan *out);
bsg_status bsg_batched_plan_run(bsg_batch_plan plan);
bsg_status bsg_batched_plan_destroy(bsg_batch_plan plan);
/* autotuner switch (0 off, 1 on, -1 on and forget the cache) and its cache:
 * entries of 6 ints (block rows, k and cols padded, digits, slots per tile,
 * stages, 0 = as many as fit) */
bsg_status bsg_ctx_set_autotune(bsg_ctx ctx, int on);
bsg_status bsg_ctx_autotune_entries(bsg_ctx ctx, int *entries, int cap, int *n);

/* ---- learned Strassen scheduling (no counterpart in the reference, whose
 *      choice is the cost model of matmult_strassen_dryrun,
 *      strassen.hpp:602-640) ----
 * Policies for the per-node choice (a node is a quadrant product of the
 * hybrid recursion, strassen.hpp:418-508):
 *   BSG_SCHED_COST   the reference's cost model (what bsg_matmult_strassen_sparse does)
 *   BSG_SCHED_NONE   no Strassen node: screened sparse recursion only
 *   BSG_SCHED_ROOT   Strassen at the root node only (block count a power of two),
 *                    recursing to min_size_for_strassen
 *   BSG_SCHED_DENSE  the root node's product as one dense tile (every block
 *                    product, unscreened)
 *   BSG_SCHED_MLP    a trained bsg_sched: per node whose blocks are all present,
 *                    the option with the smallest predicted log(t_option /
 *                    t_sparse) among Strassen-Winograd of depth 1, 2 or 3 at the
 *                    node and a dense tile, where that prediction is < 0; the
 *                    screened sparse recursion elsewhere; levels with more than
 *                    65536 nodes keep the cost model
 * A bsg_sched is a 2 x 64 MLP on BSG_SCHED_FEATURES inputs: 25 node features
 * (level, flop counts, block densities, log-norm histograms) and the option
 * one-hot (depth 1, 2, 3, dense tile), trained on the device by the library's
 * own forward / backward / Adam kernels. */
enum { BSG_SCHED_COST = 0, BSG_SCHED_NONE = 1, BSG_SCHED_ROOT = 2, BSG_SCHED_MLP = 3, BSG_SCHED_DENSE = 4 };
#define BSG_SCHED_NODE_FEATURES 25
#define BSG_SCHED_OPTIONS 4
#define BSG_SCHED_FEATURES 29
bsg_status bsg_sched_create(bsg_ctx ctx, bsg_sched *out);
bsg_status bsg_sched_destroy(bsg_sched sched);
bsg_status bsg_sched_param_count(int *out);
bsg_status bsg_sched_init(bsg_sched sched, uint64_t seed);                 /* He-uniform weights, zero biases */
bsg_status bsg_sched_set_params(bsg_sched sched, const float *params);     /* host, bsg_sched_param_count floats */
bsg_status bsg_sched_get_params(bsg_sched sched, float *params);
/* y[i] = net(x[i]), x host n x BSG_SCHED_FEATURES row-major */
bsg_status bsg_sched_predict(bsg_sched sched, const float *x, int n, float *y);
/* mean squared error of net(x) against t and its gradient (host buffers) */
bsg_status bsg_sched_loss_grad(bsg_sched sched, const float *x, const float *t, int n, float *loss, float *grad);
/* Adam on the mean squared error, minibatches of a seeded shuffle */
bsg_status bsg_sched_train(bsg_sched sched, const float *x, const float *t, int n, int epochs, int batch, float lr,
                           uint64_t seed, float *final_loss);
/* node features (BSG_SCHED_NODE_FEATURES floats) and eligibility of the root
 * node of C = A B's decision tree */
bsg_status bsg_strassen_root_features(bsg_bsm C, bsg_bsm A, bsg_bsm B, double thresh, float *features,
                                      int *eligible);
/* matmult_strassen_sparse with a scheduling policy; n_strassen_nodes (may be
 * NULL) receives the number of nodes that ran Strassen or a dense tile */
bsg_status bsg_matmult_strassen_sparse_sched(bsg_bsm C, bsg_bsm A, bsg_bsm B, double thresh,
                                             size_t min_size_for_strassen, int form, int n_digits, int policy,
                                             bsg_sched sched, uint64_t *n_strassen_nodes);

/* ---- BlockSparse3DTensor<double> = slices of BlockSparseMatrix
 *      (blocksparse3d_tensor.h:8-43; declared but never defined there) ---- */
/* C_ij = sum_l sum_k op(A^l)_ik op(B^l)_kj  (blocksparse3d_tensor.h:11-16) */
bsg_status bsg_tensormult_contract(bsg_bsm C, const bsg_bsm *A, int tA, const bsg_bsm *B, int tB, size_t n_slices,
                                   double thresh, double alpha, double beta);
/* C^l_ij = sum_k op(A)_ik op(B^l)_kj  (blocksparse3d_tensor.h:18-24), one launch over all slices */
bsg_status bsg_tensormult_batched(const bsg_bsm *C, bsg_bsm A, int tA, const bsg_bsm *B, int tB, size_t n_slices,
                                  double thresh, double alpha, double beta);

/* ---- drivers ---- */
typedef struct bsg_rik_args {
    size_t n_bf, n_aux, n_occ, n_vec2; /* occ_ri_k_step.cpp:19-22 */
    const double *ints;                /* n_vec2 x n_aux column-major, (mn|P)' compressed (:29-30) */
    const uint64_t *keys;              /* n_vec2 v2m keys, key = row + col*n_bf (:35-36) */
    const double *c_occ;               /* n_bf x n_occ column-major occupied MOs (:33-34) */
    int where;                         /* BSG_HOST or BSG_DEVICE for the three inputs */
    size_t bs;                         /* block size (:26) */
    double thresh;                     /* per-element screening threshold (:27) */
    int n_part;                        /* P partitions summed in order (OpenMP team size, :90-122) */
    int form;                          /* BSG_FORM_FP64 or BSG_FORM_OZAKI */
    int n_digits;                      /* Ozaki slices per operand (form OZAKI) */
    size_t p_chunk;                    /* aux functions per batched launch (0 = automatic) */
} bsg_rik_args;

/* occ-RI-K step (occ_ri_k_step.cpp:83-130): K_{mu j} = sum_{P,i} (mu i|P) [(ij|P)+(ji|P)],
 * K_out n_bf x n_occ column-major.  stats_out (may be NULL) receives
 * [surviving block products of the three GEMMs, mui blocks, ij blocks]. */
bsg_status bsg_rik_occ_step(bsg_ctx ctx, const bsg_rik_args *args, double *K_out, int out_where,
                            uint64_t stats_out[5]);

/* Screening state of every aux function P after an occ-RI-K step, for mask
 * parity between the arithmetic forms (host arrays, column-major blocks):
 * mui_P = U_P C block norms and presence (nb x nob per P, nb = ceil(n_bf/bs),
 * nob = ceil(n_occ/bs); a norm is meaningful where its flag is set),
 * ij_P = C^T mui_P presence, ijs_P = ij_P + ij_P^T block norms and presence
 * (nob x nob per P; the norm of a block without a transpose partner stays 0,
 * as blocksparsematrix.hpp:224-248 leaves it), and the block norms of C. */
typedef struct {
    double *mui_norm;  /* n_aux * nb * nob, index P*nb*nob + a + jb*nb */
    uint8_t *mui_flag;
    uint8_t *ij_flag;  /* n_aux * nob * nob, index P*nob*nob + ib + jb*nob */
    double *ijs_norm;
    uint8_t *ijs_flag;
    double *c_norm;    /* nb * nob, index a + jb*nb */
} bsg_rik_screen_trace;
/* bsg_rik_occ_step that also fills *trace (the screens of occ_ri_k_step.cpp:
 * 107-116: mui_P.calc_frobenius_norms() :108, ijs.add_transpose :113) */
bsg_status bsg_rik_occ_step_trace(bsg_ctx ctx, const bsg_rik_args *args, double *K_out, int out_where,
                                  uint64_t stats_out[5], const bsg_rik_screen_trace *trace);

/* Symmetric exchange matrix K_mn = sum_{P,i} mui_P(m,i) mui_P(n,i), with
 * mui_P = (mu i|P) the screened product U_P C the occ step builds
 * (occ_ri_k_step.cpp:102-108).  No counterpart in the reference, whose driver
 * stops at K_{mu j}: per P it adds matmult(Kmn_sub, mui_P, N, mui_P, T, thresh,
 * 1, 1) the way :116 adds mui_P ijs_P, partitions as in bsg_rik_occ_step.
 * Kmn_out: n_bf x n_bf column-major, exactly symmetric (lower blocks computed,
 * upper mirrored; in the FP64 form the mirror equals the computed upper block
 * bit for bit).  K_out (n_bf x n_occ, may be NULL) receives the occ step's K
 * from the same pass.  stats_out (may be NULL): bsg_rik_occ_step's five
 * counters, then the surviving block products of K_mn. */
bsg_status bsg_rik_kmn_step(bsg_ctx ctx, const bsg_rik_args *args, double *Kmn_out, double *K_out, int out_where,
                            uint64_t stats_out[6]);

/* The occ-RI-K step above without any device allocation (no counterpart in
 * the reference, which runs on the host).  For callers that cannot allocate
 * device memory: code under a framework whose caching allocator owns the
 * device heap, processes with a fixed memory budget, and latency-critical
 * streams that cannot absorb cudaFree's implicit synchronization.  Inputs
 * (args->where must be BSG_DEVICE) and K_dev (n_bf x n_occ, column-major) are
 * the caller's device buffers; FP64 form only.  All intermediates live in a
 * 32 MiB file-scope device array that every GPU loading the library keeps
 * until exit; problems whose per-aux-function workspace exceeds it are
 * rejected with BSG_ERR_ARG.  The first call on a device looks up that
 * array's address (make it before any stream capture); calls share the array,
 * so calls that overlap on the GPU race -- serialize them.  The current device
 * must own cuda_stream, K_dev and the inputs (buffers on another device are
 * rejected with BSG_ERR_ARG).  With stats_out NULL the call only enqueues its
 * kernels and does not wait for the stream; integral keys are then checked on
 * the device: a key outside the N_bf x N_bf matrix is skipped and K_dev is
 * filled with NaN.  With stats_out the call waits for its stream once, and
 * returns BSG_ERR_ARG for such a key as well.  Results equal
 * bsg_rik_occ_step's bit for bit. */
bsg_status bsg_rik_occ_step_noalloc(const bsg_rik_args *args, double *K_dev, void *cuda_stream,
                                    uint64_t stats_out[5]);

/* 3c->2c transform (3c_2c_transform.cpp:44-57): out = X * V^{-1/2} through
 * matmult on block-sparse copies (input threshold 0, out pre-filled 0).  In
 * the mixed form with where == BSG_HOST, X streams in by row ranges beside
 * the transform: pinned host memory (cudaHostAlloc / cudaHostRegister) is read
 * by 16 SMs the GEMM launches of the call leave free, other host memory goes
 * through the copy engine; the result is the same either way. */
bsg_status bsg_3c2c_transform(bsg_ctx ctx, size_t n_vec2, size_t n_aux, const double *ints_3c,
                              const double *v_m12, int where, size_t bs, double thresh, int form, int n_digits,
                              double *out, int out_where);
/* the same, with the number of surviving block products in *nsig_out (the
 * screen uses the FP64 block norms of X and V^{-1/2} in both forms) */
bsg_status bsg_3c2c_transform_nsig(bsg_ctx ctx, size_t n_vec2, size_t n_aux, const double *ints_3c,
                                   const double *v_m12, int where, size_t bs, double thresh, int form, int n_digits,
                                   double *out, int out_where, uint64_t *nsig_out);

#ifdef __cplusplus
}
#endif
#endif
