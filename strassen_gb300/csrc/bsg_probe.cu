// FP64 FMA throughput probe: the denominator of the FP64 roofline (the
// measured peaks file of this machine covers HBM and bf16 only).
#include "bsg_internal.cuh"

namespace bsg {

__global__ void k_dfma_probe(double *out, int iters, double a, double b) {
    double x[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = (double)(threadIdx.x + j);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) x[j] = fma(x[j], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += x[j];
    if (s == 12345.678) out[0] = s;  // keeps the chains alive
}

}  // namespace bsg

using namespace bsg;

extern "C" bsg_status bsg_probe_fp64_peak(bsg_ctx ctx, double *gflops) {
    return guard([&] {
        BSG_REQUIRE(ctx && gflops, BSG_ERR_ARG, "NULL argument");
        cudaStream_t s = ctx->stream;
        DevBuf o(8, s);
        cudaEvent_t e0, e1;
        BSG_CUDA(cudaEventCreate(&e0));
        BSG_CUDA(cudaEventCreate(&e1));
        const int blocks = ctx->sm_count * 4, threads = 256, iters = 4096;
        k_dfma_probe<<<blocks, threads, 0, s>>>(o.as<double>(), 64, 0.999, 1e-3);  // warm-up
        BSG_CUDA(cudaEventRecord(e0, s));
        k_dfma_probe<<<blocks, threads, 0, s>>>(o.as<double>(), iters, 0.999, 1e-3);
        BSG_CUDA(cudaEventRecord(e1, s));
        ctx->note_launch(2);
        BSG_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        BSG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        *gflops = 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e9;
    });
}
