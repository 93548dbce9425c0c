// RI-K pipeline shared declarations.
#pragma once
#include "bsg_internal.cuh"

namespace bsg {

// device-resident inputs of one RI-K step
struct RikDev {
    size_t n_bf = 0, n_aux = 0, n_occ = 0, n_vec2 = 0, bs = 0, p_chunk = 0;
    const double *ints = nullptr;
    const uint64_t *keys = nullptr;
    const double *c_occ = nullptr;
    double thresh = 0.0;
    int n_part = 1;
    int n_digits = 4;
};

void rik_fp64(bsg_ctx ctx, const RikDev &d, double *K_dev, uint64_t stats[5]);
void rik_ozaki(bsg_ctx ctx, const RikDev &d, double *K_dev, uint64_t stats[5]);

}  // namespace bsg
