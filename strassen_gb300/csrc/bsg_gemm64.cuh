// Grouped FP64 block-product machinery shared by matmult, the 3-index tensor
// contractions, the Strassen leaves and the RI-K pipeline.
#pragma once
#include "bsg_internal.cuh"

namespace bsg {

// One output block of a grouped launch.
struct GemmItem {
    double *c;        // output block (column-major, ld = rows)
    double *c_norm;   // cached norm slot (set to 0 when the block is fresh), may be null
    int rows, cols;
    int fresh;        // 1: block was created by this product (first pair assigns)
    uint32_t p0, p1;  // pair range
};

// One block product contributing to an item, in accumulation order.
struct GemmPair {
    const double *a;  // stored A block (column-major, ld = lda)
    const double *b;  // stored B block (column-major, ld = ldb)
    int k;            // contraction extent
    int lda, ldb;
};

// C_item = alpha*sum_pairs op(A)op(B) (+ C_item unless fresh), each pair an
// fma chain over k from 0 followed by C = alpha*t + C; bit-identical to the
// deterministic BLAS definition.
void launch_gemm64(bsg_ctx ctx, const GemmItem *d_items, size_t n_items, const GemmPair *d_pairs, int tA, int tB,
                   double alpha, int max_rows, int max_cols, cudaStream_t s);

// geometry of a screened product op(A) (ni x nk) * op(B) (nk x nj)
struct ScreenGeom {
    int tA, tB;
    size_t nib, njb, nkb, ibs, jbs, kbs, ni, nj, nk;
    double tpb;
};

// Screened block-triple enumeration for matmult and the 3-index tensor
// products.  A "slice" is one (A, B) operand pair; an output matrix sums the
// slices in [lo, hi) (contract) or exactly one slice (batched).
struct SliceOps {
    double *const *a;
    const double *an;
    size_t a_nrb;
    double *const *b;
    const double *bn;
    size_t b_nrb;
};

// Runs C_out[c] = alpha * sum over slices [lo[c], hi[c]) and surviving
// block triples + beta*C_out[c] with the reference's matmult semantics
// (blocksparsematrix.hpp:293-414).  Returns the number of surviving triples.
uint64_t screened_product(bsg_ctx ctx, const std::vector<bsg_bsm> &Cs, const std::vector<bsg_bsm> &As, int tA,
                          const std::vector<bsg_bsm> &Bs, int tB, const std::vector<std::pair<size_t, size_t>> &ranges,
                          double thresh, double alpha, double beta, int form, int n_digits);

// Screening of one product C = alpha op(A) op(B) + beta C (single slice):
// geometry, beta handling, surviving-pair counts, the C blocks that become
// non-empty (allocated; fresh blocks get their first product assigned) and
// the output items, column-major block order.
struct ScreenItems {
    ScreenGeom g;
    std::vector<GemmItem> items;
    std::vector<uint32_t> item_ib, item_jb;
    uint64_t total = 0;  // surviving block triples
};
ScreenItems screen_items(bsg_ctx ctx, bsg_bsm C, bsg_bsm A, int tA, bsg_bsm B, int tB, double thresh, double beta);

}  // namespace bsg
