// Ozaki-style split-precision block products on tcgen05 tensor cores.
#include "bsg_ozaki.cuh"

namespace bsg {

void ozaki_grouped_gemm(bsg_ctx, const std::vector<GemmItem> &, const GemmItem *, const GemmPair *, uint64_t, int, int,
                        double, int, int, size_t, int, cudaStream_t) {
    throw Error{BSG_ERR_UNSUPPORTED, "Ozaki form not available"};
}

}  // namespace bsg

#include "bsg_rik.cuh"
namespace bsg {
void rik_ozaki(bsg_ctx, const RikDev &, double *, uint64_t *) {
    throw Error{BSG_ERR_UNSUPPORTED, "Ozaki RI-K form not available"};
}
}  // namespace bsg
