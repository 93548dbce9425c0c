// Ozaki-style split-precision block products on tcgen05 tensor cores.
#pragma once
#include "bsg_gemm64.cuh"

namespace bsg {

// Grouped block products of a screened_product call in the Ozaki form: the
// same items / pairs (and so the same screening masks) as the FP64 form.
void ozaki_grouped_gemm(bsg_ctx ctx, const std::vector<GemmItem> &items, const GemmItem *d_items,
                        const GemmPair *d_pairs, uint64_t n_pairs, int tA, int tB, double alpha, int max_r, int max_c,
                        size_t kbs, int n_digits, cudaStream_t s);

}  // namespace bsg
