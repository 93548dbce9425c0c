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
    // optional screen trace (device arrays of every aux function P, NULL =
    // off), written per chunk: mui_P block norms and flags (nb x nob, index
    // P*nb*nob + a + jb*nb), ij_P flags, ijs_P block norms and flags (nob x
    // nob, index P*nob*nob + ib + jb*nob), and the C block norms (nb x nob)
    double *tr_mui_norm = nullptr;
    uint8_t *tr_mui_flag = nullptr;
    uint8_t *tr_ij_flag = nullptr;
    double *tr_ijs_norm = nullptr;
    uint8_t *tr_ijs_flag = nullptr;
    double *tr_c_norm = nullptr;
};

// copies one chunk's screening state (aux functions P0 .. P0+np) into the trace
void rik_trace_chunk(const RikDev &d, size_t P0, size_t np, const double *mnorm, const uint8_t *mflag,
                     const uint8_t *ijflag, const double *snorm, const uint8_t *sflag, cudaStream_t s);

// K_dev (n_bf x n_occ) and Kmn_dev (n_bf x n_bf) may each be NULL (that
// output is skipped); stats: the five occ-step counters and the K_mn products
void rik_fp64(bsg_ctx ctx, const RikDev &d, double *K_dev, double *Kmn_dev, uint64_t stats[6]);

// stage kernels shared by the FP64 and Ozaki pipelines (bsg_rik.cu)
__global__ void k_scatter(const double *__restrict__ ints, const uint64_t *__restrict__ keys, size_t n_vec2,
                          size_t P0, size_t u_stride, double *__restrict__ U);
__global__ void k_unorms(const double *__restrict__ U, size_t n_bf, size_t bs, size_t nb, size_t n_p, double tpb,
                         double *__restrict__ norm, uint8_t *__restrict__ flag);
__global__ void k_ijs(const double *__restrict__ ij, const uint8_t *__restrict__ ijflag, size_t n_occ, size_t bs,
                      size_t nob, double *__restrict__ ijs, double *__restrict__ snorm, uint8_t *__restrict__ sflag);
__global__ void k_cnorms(const double *__restrict__ C, size_t n_bf, size_t n_occ, size_t bs, size_t nb, size_t nob,
                         double *__restrict__ cnorm);
void rik_ozaki(bsg_ctx ctx, const RikDev &d, double *K_dev, double *Kmn_dev, uint64_t stats[6]);
// dense device 3c->2c in the Ozaki form (bsg_3c2c_oz.cu)
void transform_3c2c_ozaki(bsg_ctx ctx, size_t n_vec2, size_t n_aux, const double *X, const double *V, size_t bs,
                          double thresh, int n_digits, double *out, uint64_t *nsig_out);
// the same with X in host memory: uploaded in row ranges that overlap the
// transform of the previous range (V and out on the device)
void transform_3c2c_ozaki_upload(bsg_ctx ctx, size_t n_vec2, size_t n_aux, const double *X_host, const double *V,
                                 size_t bs, double thresh, int n_digits, double *out, uint64_t *nsig_out);

}  // namespace bsg
